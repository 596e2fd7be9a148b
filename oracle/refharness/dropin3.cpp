/* dropin3.cpp -- the drop-in test for dSim3: the reference's own SpinSystem
 * (dSim3/src/spinSystem.cpp, the scratch copy prepared by oracle/build_ref.py)
 * constructed with useGpu = true and linked against this project's
 * libdsim3.so in place of the reference's spinSystem.cu.  It runs the calls
 * of dSim3/src/diffusion.cpp:1118-1153 (initFibers, populateCubes,
 * constructAllRTrees, build, resetSpins), so every device allocation, copy,
 * binding and copyConstantToDevice comes from the reference's code; then
 * updateSpins takes the reference's GPU branch (spinSystem.cpp:1942-1963) with
 * the steps replayed from a file (dsim3_set_replay), and the arrays are
 * dumped for the oracle comparison.  Test infrastructure only.
 *
 * args: mesh= out= N= seed= spaceScale= dt= extraAdc= myelinAdc= intraAdc=
 *       perm= extraT2= myelinT2= intraT2= startBox= gx= gy= gz= gamma=
 *       iters= reflType= draws=<float32 [iters][N][4]> */
#include <ctime>
#include "dump.h"
#include <vector>
#include "spinSystem.h"
#include "spinSystem.cuh"

extern "C" {
void dsim3_set_replay(const float* draws, unsigned int* counts);
int dsim3_last_status(void);
const char* dsim3_last_error(void);
unsigned int dsim3_status(void);
}

class DropIn : public SpinSystem {
public:
    DropIn(int n, float ss, float gam, uint refl, float ea, float ma, float ia, float p, float et2,
           float mt2, float it2, float dt, float sb)
        : SpinSystem(n, true, ss, gam, false, 0, refl, ea, ma, ia, p, et2, mt2, it2, dt, sb) {}
    void dumpAll(FILE* f, const char* sfx) {
        std::string s(sfx);
        dump_rec(f, ("pos" + s).c_str(), "f4", m_hPos, (uint64_t)m_numSpins * 3, 4);
        dump_rec(f, ("spins" + s).c_str(), "u1", m_hSpins, (uint64_t)m_numSpins * sizeof(spinData), 1);
    }
    void dumpSubstrate(FILE* f) {
        dump_rec(f, "vertices", "f4", m_vertices, (uint64_t)m_nVertices * 3, 4);
        dump_rec(f, "trgls", "u4", m_trgls, (uint64_t)m_nTriangles * 3, 4);
        dump_rec(f, "triInfo", "u4", m_hTriInfo, (uint64_t)m_nTriangles * 3, 4);
        dump_rec(f, "helpers", "f4", m_triangleHelpers, (uint64_t)m_nTriangles * 12, 4);
        uint32_t g[3] = {m_numCubes, m_totalNumCubes, m_maxTrianglesPerCube};
        dump_rec(f, "grid", "u4", g, 3, 4);
        dump_rec(f, "cubeCounter", "u4", m_hCubeCounter, m_totalNumCubes, 4);
        dump_rec(f, "trianglesInCubes", "u4", m_hTrianglesInCubes,
                 (uint64_t)m_totalNumCubes * m_maxTrianglesPerCube, 4);
        dump_rec(f, "stdDevs", "f4", m_hStdDevs, 4, 4);
        dump_rec(f, "T2", "f4", m_hT2Values, 4, 4);
    }
};

int main(int argc, char** argv) {
    auto kv = parse_kv(argc, argv);
    int N = (int)kvd(kv, "N", 1000);
    uint iters = (uint)kvd(kv, "iters", 10);
    DropIn* h = new DropIn(N, (float)kvd(kv, "spaceScale", 60), (float)kvd(kv, "gamma", 42576.0),
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
    // the replayed steps, on the device through the reference's own ABI calls
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
    h->dumpAll(f, "0");
    float3 g = make_float3((float)kvd(kv, "gx", 0), (float)kvd(kv, "gy", 0), (float)kvd(kv, "gz", 0));
    h->setGradient(g);
    dsim3_set_replay(dDraws, dCnt);
    h->updateSpins((float)kvd(kv, "dt", 0.005), iters);
    dsim3_set_replay(nullptr, nullptr);
    h->getArray();
    h->getSpinArray();
    copyArrayFromDevice(cnt.data(), dCnt, 0, (int)(cnt.size() * 4));
    h->dumpAll(f, "1");
    dump_rec(f, "counts", "u4", cnt.data(), cnt.size(), 4);
    int32_t st[2] = {dsim3_last_status(), (int32_t)dsim3_status()};
    dump_rec(f, "status", "i4", st, 2, 4);
    fclose(f);
    if (st[0] != 0) fprintf(stderr, "%s\n", dsim3_last_error());
    return st[0] != 0 ? 4 : 0;  /* no delete: the reference destructor frees arrays twice */
}
