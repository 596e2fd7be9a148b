/* harness2.cpp -- drives the reference's own dSim2 CPU path (compiled from
 * dSim2/src/spinSystem.cpp by oracle/build_ref.py) as
 * dSim2/src/diffusion.cpp does (initFibers(FILE*), build, reset), then dumps
 * the arrays the GPU cylinder engine is checked against.  Test
 * infrastructure only.
 * args: fibers= out= N= seed= spaceScale= dt= extraAdc= intraAdc= myelinAdc=
 *       extraT2= intraT2= myelinT2= perm= inner= gx= gy= gz= gamma= iters= */
#include <ctime>
#include "dump.h"
#include "spinSystem.h"

class Harness : public SpinSystem {
public:
    Harness(int n, float ss, float gam) : SpinSystem(n, false, ss, gam, false) {}
    void dumpAll(FILE* f, const char* sfx) {
        std::string s(sfx);
        dump_rec(f, ("pos" + s).c_str(), "f4", m_hPos, (uint64_t)m_numSpins * 4, 4);
        dump_rec(f, ("seed" + s).c_str(), "u4", m_hSeed, (uint64_t)m_numSpins * 4, 4);
        dump_rec(f, ("params" + s).c_str(), "f4", m_hPartParams, (uint64_t)m_numSpins * m_nParams, 4);
    }
    void dumpSubstrate(FILE* f) {
        dump_rec(f, "fiberPos", "f4", m_fiberPos, (uint64_t)m_numFibers * 4, 4);
        float mr = m_maxFiberRadius;
        dump_rec(f, "maxR", "f4", &mr, 1, 4);
        uint32_t g[3] = {m_numCubes, m_totalNumCubes, m_maxFibersPerCube};
        dump_rec(f, "grid", "u4", g, 3, 4);
        dump_rec(f, "cubeLength", "f4", &m_cubeLength, 1, 4);
        dump_rec(f, "cubeCounter", "u4", m_hCubeCounter, m_totalNumCubes, 4);
        dump_rec(f, "cubes", "u4", m_hCubes, (uint64_t)m_totalNumCubes * m_maxFibersPerCube, 4);
    }
};

int main(int argc, char** argv) {
    auto kv = parse_kv(argc, argv);
    int N = (int)kvd(kv, "N", 1000);
    Harness* h = new Harness(N, (float)kvd(kv, "spaceScale", 20), (float)kvd(kv, "gamma", 42576.0));
    srand((unsigned)kvd(kv, "seed", 1));
    FILE* fp = fopen(kv["fibers"].c_str(), "r");
    if (!fp) { perror("fibers"); return 2; }
    h->initFibers(fp, (float)kvd(kv, "inner", 1.0));
    fclose(fp);
    h->setAdc((float)kvd(kv, "extraAdc", 2.0), (float)kvd(kv, "intraAdc", 2.0), (float)kvd(kv, "myelinAdc", 0.1));
    h->setT2((float)kvd(kv, "extraT2", 80), (float)kvd(kv, "intraT2", 80), (float)kvd(kv, "myelinT2", 7.5));
    h->setPermeability((float)kvd(kv, "perm", 0.0));
    if (!h->build()) { fprintf(stderr, "build() failed\n"); return 3; }
    h->reset(SpinSystem::CONFIG_RANDOM);
    FILE* f = fopen(kv["out"].c_str(), "wb");
    h->dumpSubstrate(f);
    h->dumpAll(f, "0");
    float3 g = make_float3((float)kvd(kv, "gx", 0), (float)kvd(kv, "gy", 0), (float)kvd(kv, "gz", 0));
    h->setGradient(g);
    uint iters = (uint)kvd(kv, "iters", 10);
    double t0 = now_ms();
    h->update((float)kvd(kv, "dt", 0.01), iters);
    double ms = now_ms() - t0;
    h->dumpAll(f, "1");
    double sig = h->getMrSignal();
    dump_rec(f, "signal", "f8", &sig, 1, 8);
    dump_rec(f, "update_ms", "f8", &ms, 1, 8);
    fclose(f);
    return 0;
}
