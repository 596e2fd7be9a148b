/* seq2.cpp -- runs the reference's own dSim2 PGSE sequencer and results
 * writer: update() and the results-file header of dSim2/src/diffusion.cpp
 * (diffusion2_types.inc, diffusion2_update.inc and diffusion2_header.inc,
 * taken unchanged by oracle/build_ref.py).  This file defines the globals they
 * use and stands in for the SpinSystem that update() drives: it records every
 * call (reset, gradient, update) and answers getMrSignal with given signals,
 * one per gradient run.  update() is called until the sequence is done; the
 * reference's update() then writes its timing lines, closes the results file
 * and calls exit(0), and the recording is written by an exit handler.  Test
 * infrastructure only.
 *
 * args: grads=<float32 [n][6]> signals=<float64 [n]> timestep= iterations=
 *       numSpins= spaceScale= radiusMean= spacingMean= crossFraction= useGpu=
 *       fiberFile= outm=<results file> out=<dump> */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "dump.h"

typedef unsigned int uint;
struct float3 { float x, y, z; };
static inline float3 operator*(float3 a, float s) { float3 r = {a.x * s, a.y * s, a.z * s}; return r; }

// stands in for SpinSystem: the calls update() makes, recorded
class SpinSystem {
public:
    enum SpinConfig { CONFIG_RANDOM, CONFIG_GRID, _NUM_CONFIGS };
    std::vector<double> sig;   // [run] signals returned at each read
    std::vector<float> calls;  // per update: reads so far, resets so far, gx, gy, gz, dt, iterations
    std::vector<float> events; // pairs {1 reset | 2 read, update calls before it}
    uint reads = 0, resets = 0, steps = 0;
    float3 g = {0.0f, 0.0f, 0.0f};
    double getMrSignal() {
        const double s = reads < sig.size() ? sig[reads] : 0.0;
        reads++;
        events.push_back(2.0f);
        events.push_back((float)(calls.size() / 7));
        return s;
    }
    void reset(SpinConfig) {
        resets++;
        events.push_back(1.0f);
        events.push_back((float)(calls.size() / 7));
    }
    void setGradient(float3 G) { g = G; }
    float update(float dt, uint iterations) {
        const float rec[7] = {(float)reads, (float)resets, g.x, g.y, g.z, dt, (float)iterations};
        calls.insert(calls.end(), rec, rec + 7);
        steps += iterations;
        return 0.001f;
    }
    uint getNumTimeSteps() { return steps; }
};

SpinSystem* psystem = 0;
FILE* outFilePtr = NULL;
uint stepCount = 0;
float timestep = 0.005f;
int iterations = 1;
float totalKernelTime = 0.0f;
float time_in_sec = 0.0f;
float curStepsPerSec = 0.0f;

#include "diffusion2_types.inc"
gradStruct* gGrads = NULL;
#include "diffusion2_update.inc"

// the header main() writes when the results file is named (the statements
// between its fopen and the fibers line, unchanged)
static void write_header(char* outFilename, float fiberRadius, float fiberSpace, float spaceScale, uint numSpins,
                         float crossFraction, bool useGpu, const char* fiberFileConst) {
#include "diffusion2_header.inc"
}

static SpinSystem rec;
static std::string dumpPath;

static void write_dump() {
    FILE* f = fopen(dumpPath.c_str(), "wb");
    if (!f) return;
    dump_rec(f, "calls", "f4", rec.calls.data(), rec.calls.size(), 4);
    dump_rec(f, "events", "f4", rec.events.data(), rec.events.size(), 4);
    fclose(f);
}

template <typename T>
static std::vector<T> read_all(const std::string& path) {
    std::vector<T> v;
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) { perror(path.c_str()); exit(2); }
    T x;
    while (fread(&x, sizeof(T), 1, f) == 1) v.push_back(x);
    fclose(f);
    return v;
}

int main(int argc, char** argv) {
    auto kv = parse_kv(argc, argv);
    std::vector<float> rows = read_all<float>(kv["grads"]);
    rec.sig = read_all<double>(kv["signals"]);
    const uint numGrads = (uint)(rows.size() / 6);
    // the gradient list, linked as main() links the rows of the .grads file
    gradStruct* prev = NULL;
    for (uint i = 0; i < numGrads; i++) {
        gradStruct* g = new gradStruct;
        g->lDelta = rows[6 * i]; g->bDelta = rows[6 * i + 1]; g->readOut = rows[6 * i + 2];
        g->gx = rows[6 * i + 3]; g->gy = rows[6 * i + 4]; g->gz = rows[6 * i + 5];
        g->next = NULL;
        if (prev) prev->next = g; else gGrads = g;
        prev = g;
    }
    timestep = (float)kvd(kv, "timestep", 0.005);
    iterations = (int)kvd(kv, "iterations", 1);
    std::string ff = kv["fiberFile"], om = kv["outm"];
    dumpPath = kv["out"];
    write_header((char*)om.c_str(), (float)kvd(kv, "radiusMean", 1.0), (float)kvd(kv, "spacingMean", 0.2),
                 (float)kvd(kv, "spaceScale", 100.0), (uint)kvd(kv, "numSpins", 20000),
                 (float)kvd(kv, "crossFraction", 0.0), kvd(kv, "useGpu", 1.0) != 0.0, ff.c_str());
    psystem = &rec;
    atexit(write_dump);
    for (uint k = 0; k < 50000000u; k++) update();   // update() exits when the sequence is done
    fprintf(stderr, "sequence did not finish\n");
    return 3;
}
