/* harness3.cpp -- drives the reference's own dSim3 CPU path (compiled from
 * dSim3/src/spinSystem.cpp by oracle/build_ref.py) through the same calls
 * dSim3/src/diffusion.cpp:1118-1153 makes, then dumps every array the GPU
 * engine is checked against.  Test infrastructure only.
 *
 * args: mesh= out= N= seed= spaceScale= dt= extraAdc= myelinAdc= intraAdc=
 *       perm= extraT2= myelinT2= intraT2= startBox= gx= gy= gz= gamma=
 *       iters= reflType= [init=<state file: pos f32[3N], seed u32[2N], spinData[N]>]
 *       [threads=<n>: time updateSpins only]  */
#include <ctime>
#include "dump.h"
#include "spinSystem.h"

class Harness : public SpinSystem {
public:
    Harness(int n, float ss, float gam, uint refl, float ea, float ma, float ia, float p, float et2,
            float mt2, float it2, float dt, float sb)
        : SpinSystem(n, false, ss, gam, false, 0, refl, ea, ma, ia, p, et2, mt2, it2, dt, sb) {}
    void dumpAll(FILE* f, const char* sfx) {
        std::string s(sfx);
        dump_rec(f, ("pos" + s).c_str(), "f4", m_hPos, (uint64_t)m_numSpins * 3, 4);
        dump_rec(f, ("seed" + s).c_str(), "u4", m_hSeed, (uint64_t)m_numSpins * 2, 4);
        dump_rec(f, ("spins" + s).c_str(), "u1", m_hSpins, (uint64_t)m_numSpins * sizeof(spinData), 1);
    }
    void dumpSubstrate(FILE* f) {
        uint32_t c[7] = {m_nVertices, m_nTriangles, m_nFibers, m_nAxonFibers, m_nMyelinFibers,
                         m_nGliaFibers, m_maxTrianglesOnSurface};
        dump_rec(f, "counts", "u4", c, 7, 4);
        dump_rec(f, "vertices", "f4", m_vertices, (uint64_t)m_nVertices * 3, 4);
        dump_rec(f, "trgls", "u4", m_trgls, (uint64_t)m_nTriangles * 3, 4);
        dump_rec(f, "triInfo", "u4", m_hTriInfo, (uint64_t)m_nTriangles * 3, 4);
        dump_rec(f, "helpers", "f4", m_triangleHelpers, (uint64_t)m_nTriangles * 12, 4);
        float mx[3] = {m_xmax, m_ymax, m_zmax};
        dump_rec(f, "maxabs", "f4", mx, 3, 4);
        uint32_t g[3] = {m_numCubes, m_totalNumCubes, m_maxTrianglesPerCube};
        dump_rec(f, "grid", "u4", g, 3, 4);
        dump_rec(f, "cubeLength", "f4", &m_cubeLength, 1, 4);
        dump_rec(f, "cubeCounter", "u4", m_hCubeCounter, m_totalNumCubes, 4);
        dump_rec(f, "trianglesInCubes", "u4", m_hTrianglesInCubes,
                 (uint64_t)m_totalNumCubes * m_maxTrianglesPerCube, 4);
        dump_rec(f, "stdDevs", "f4", m_hStdDevs, 4, 4);
        dump_rec(f, "T2", "f4", m_hT2Values, 4, 4);
    }
    void loadState(const char* path) {
        FILE* f = fopen(path, "rb");
        if (!f) { perror(path); exit(2); }
        size_t n = m_numSpins;
        if (fread(m_hPos, 4, 3 * n, f) != 3 * n || fread(m_hSeed, 4, 2 * n, f) != 2 * n ||
            fread(m_hSpins, sizeof(spinData), n, f) != n) { fprintf(stderr, "short state\n"); exit(2); }
        fclose(f);
        setArray();
        setSpinArray();
    }
};

int main(int argc, char** argv) {
    auto kv = parse_kv(argc, argv);
    int N = (int)kvd(kv, "N", 1000);
    Harness* h = new Harness(N, (float)kvd(kv, "spaceScale", 60), (float)kvd(kv, "gamma", 42576.0),
                             (uint)kvd(kv, "reflType", 1), (float)kvd(kv, "extraAdc", 2.1),
                             (float)kvd(kv, "myelinAdc", 0.1), (float)kvd(kv, "intraAdc", 2.1),
                             (float)kvd(kv, "perm", 0.0), (float)kvd(kv, "extraT2", 80),
                             (float)kvd(kv, "myelinT2", 7.5), (float)kvd(kv, "intraT2", 80),
                             (float)kvd(kv, "dt", 0.005), (float)kvd(kv, "startBox", 0.6));
    srand((unsigned)kvd(kv, "seed", 1));
    std::string mesh = kv["mesh"];
    h->initFibers((char*)mesh.c_str());
    h->populateCubes();
    h->constructAllRTrees();
    h->build();
    h->resetSpins();
    if (kv.count("init")) h->loadState(kv["init"].c_str());
    FILE* f = fopen(kv["out"].c_str(), "wb");
    h->dumpSubstrate(f);
    h->dumpAll(f, "0");
    float3 g = make_float3((float)kvd(kv, "gx", 0), (float)kvd(kv, "gy", 0), (float)kvd(kv, "gz", 0));
    h->setGradient(g);
    uint iters = (uint)kvd(kv, "iters", 10);
    float dt = (float)kvd(kv, "dt", 0.005);
    double t0 = now_ms();
    h->updateSpins(dt, iters);
    double ms = now_ms() - t0;
    h->getArray();
    h->getSpinArray();
    h->dumpAll(f, "1");
    double sig[5];
    h->getMrSignal(sig);
    dump_rec(f, "signal", "f8", sig, 5, 8);
    dump_rec(f, "update_ms", "f8", &ms, 1, 8);
    fclose(f);
    return 0;  /* no delete: the reference destructor frees arrays twice */
}
