/* dropin2.cpp -- the drop-in test for dSim2: the reference's own SpinSystem
 * (dSim2/src/spinSystem.cpp, the scratch copy prepared by oracle/build_ref.py)
 * constructed with useGpu = true and linked against this project's
 * libdsim2.so in place of the reference's spinSystem.cu.  It runs
 * dSim2/src/diffusion.cpp's set-up (initFibers(FILE*), build, reset), so the
 * device arrays, the fiber list and the cube lists are allocated, copied and
 * bound by the reference's code; update() then takes the reference's GPU
 * branch (dSim2/src/spinSystem.cpp:857-895) with the steps replayed from a file
 * (dsim2_set_replay).  Test infrastructure only.
 *
 * args: fibers= out= N= seed= spaceScale= dt= extraAdc= intraAdc= myelinAdc=
 *       extraT2= intraT2= myelinT2= perm= inner= gx= gy= gz= gamma= iters=
 *       draws=<float32 [iters][N][4]> */
#include <ctime>
#include <vector>
#include "dump.h"
#include <vector>
#include "spinSystem.h"
#include "spinSystem.cuh"

extern "C" {
void dsim2_set_replay(const float* draws, unsigned int* counts);
int dsim2_last_status(void);
const char* dsim2_last_error(void);
unsigned int dsim2_status(void);
}

class DropIn : public SpinSystem {
public:
    DropIn(int n, float ss, float gam) : SpinSystem(n, true, ss, gam, false) {}
    void dumpHost(FILE* f, const char* sfx) {
        std::string s(sfx);
        dump_rec(f, ("pos" + s).c_str(), "f4", m_hPos, (uint64_t)m_numSpins * 4, 4);
        dump_rec(f, ("seed" + s).c_str(), "u4", m_hSeed, (uint64_t)m_numSpins * 4, 4);
        dump_rec(f, ("params" + s).c_str(), "f4", m_hPartParams, (uint64_t)m_numSpins * m_nParams, 4);
    }
    void dumpDevice(FILE* f) {
        std::vector<float> p((size_t)m_numSpins * 4);
        std::vector<uint32_t> sd((size_t)m_numSpins * 4);
        getArray();  // the positions (and phase in w) back from the device, as the reference reads them
        dump_rec(f, "pos1", "f4", m_hPos, (uint64_t)m_numSpins * 4, 4);
        copyArrayFromDevice(sd.data(), m_dSeed[m_currentSeedRead], 0, (int)(sd.size() * 4));
        dump_rec(f, "seed1", "u4", sd.data(), sd.size(), 4);
    }
    void dumpSubstrate(FILE* f) {
        dump_rec(f, "fiberPos", "f4", m_fiberPos, (uint64_t)m_numFibers * 4, 4);
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
    uint iters = (uint)kvd(kv, "iters", 10);
    DropIn* h = new DropIn(N, (float)kvd(kv, "spaceScale", 20), (float)kvd(kv, "gamma", 42576.0));
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
    std::vector<float> d((size_t)iters * N * 4);
    FILE* fd = fopen(kv["draws"].c_str(), "rb");
    if (!fd || fread(d.data(), 4, d.size(), fd) != d.size()) { fprintf(stderr, "draws file\n"); return 2; }
    fclose(fd);
    float* dDraws = nullptr;
    unsigned int* dCnt = nullptr;
    allocateArray((void**)&dDraws, (int)(d.size() * 4));
    copyArrayToDevice(dDraws, d.data(), 0, (int)(d.size() * 4));
    std::vector<unsigned int> cnt((size_t)2 * N, 0u);
    allocateArray((void**)&dCnt, (int)(cnt.size() * 4));
    copyArrayToDevice(dCnt, cnt.data(), 0, (int)(cnt.size() * 4));
    FILE* f = fopen(kv["out"].c_str(), "wb");
    h->dumpSubstrate(f);
    h->dumpHost(f, "0");
    float3 g = make_float3((float)kvd(kv, "gx", 0), (float)kvd(kv, "gy", 0), (float)kvd(kv, "gz", 0));
    h->setGradient(g);
    dsim2_set_replay(dDraws, dCnt);
    h->update((float)kvd(kv, "dt", 0.01), iters);
    dsim2_set_replay(nullptr, nullptr);
    h->dumpDevice(f);
    copyArrayFromDevice(cnt.data(), dCnt, 0, (int)(cnt.size() * 4));
    dump_rec(f, "counts", "u4", cnt.data(), cnt.size(), 4);
    int32_t st[2] = {dsim2_last_status(), (int32_t)dsim2_status()};
    dump_rec(f, "status", "i4", st, 2, 4);
    fclose(f);
    if (st[0] != 0) fprintf(stderr, "%s\n", dsim2_last_error());
    return st[0] != 0 ? 4 : 0;
}
