/* seq3.cpp -- runs the reference's own PGSE sequencer, results writer and
 * tensor fit: update() and computeTensor() of dSim3/src/diffusion.cpp
 * (diffusion_parts.inc, taken unchanged by oracle/build_ref.py), compiled
 * with the reference's vendored JAMA/TNT headers.  This file defines the
 * globals those functions use and stands in for the SpinSystem that update()
 * drives: it records every call (reset, gradient, updateSpins) and answers
 * getMrSignal with given signals, one row of 5 per gradient run.  update() is
 * called until the sequence is done, as the reference's idle loop calls it;
 * the writer appends its results file; computeTensor is then run for every
 * signal column.  Test infrastructure only.
 *
 * args: grads=<float32 [n][6]> signals=<float64 [n][5]> timeStep= stepsPerUpdate=
 *       numSpins= gamma= extraAdc= intraAdc= myelinAdc= spaceScale= permeability=
 *       fiberFile= outm=<results file> out=<dump> */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "dump.h"
#include "jama_eig.h"
#include "jama_svd.h"
#include "tnt_array1d.h"
#include "tnt_array2d.h"
#include "tnt_array2d_utils.h"

typedef unsigned int uint;
struct float3 { float x, y, z; };
static inline float3 operator*(float3 a, float s) { float3 r = {a.x * s, a.y * s, a.z * s}; return r; }

// stands in for SpinSystem: the calls update() makes, recorded
class Recorder {
public:
    std::vector<double> sig;   // [run][5] signals returned at each read
    std::vector<float> calls;  // per updateSpins: reads so far, resets so far, gx, gy, gz, dt, iterations
    std::vector<float> events; // pairs {1 reset | 2 read, updateSpins calls before it}
    uint reads = 0, resets = 0;
    float3 g = {0.0f, 0.0f, 0.0f};
    uint getNumCompartments() { return 4; }
    double getMrSignal() { return 1.0; }
    void getMrSignal(double out[]) {
        for (int c = 0; c < 5; c++) out[c] = sig[5 * (size_t)reads + c];
        reads++;
        events.push_back(2.0f);
        events.push_back((float)(calls.size() / 7));
    }
    void resetSpins() {
        resets++;
        events.push_back(1.0f);
        events.push_back((float)(calls.size() / 7));
    }
    void setGradient(float3 G) { g = G; }
    float updateSpins(float dt, uint iterations) {
        const float rec[7] = {(float)reads, (float)resets, g.x, g.y, g.z, dt, (float)iterations};
        calls.insert(calls.end(), rec, rec + 7);
        return 0.0f;
    }
};

struct _gradStruct;
typedef struct _gradStruct gradStruct;
gradStruct* gGrads = NULL;
char* fiberFile = NULL;
char* outFileName = NULL;
FILE* outFilePtr;
Recorder* psystem = 0;
uint stepCount = 0;
uint updateCount = 0;
float* gradientDataResults;
uint numOutputs;
uint numGrads = 0;
bool computedOutput = 0;
float ell1, ell2, ell3, ex, ey, ez, theta;
float timeStep = 0.01;
int stepsPerUpdate = 1;
bool useGpu = true;
bool useDisplay = false;
bool writeOut = true;
uint numSpins = 30000;
float gyroMagneticRatio = 42576.0f;
float extraAdc = 2.1, intraAdc = 2.1, myelinAdc = 0.1;
float spaceScale = 100.0f;
float permeability = 0.000002;

#include "diffusion_parts.inc"

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
    Recorder rec;
    rec.sig = read_all<double>(kv["signals"]);
    numGrads = (uint)(rows.size() / 6);
    if (rec.sig.size() < 5 * (size_t)numGrads) { fprintf(stderr, "signals\n"); return 2; }
    // the gradient list, linked as readInputs links the rows of the .grads file
    gradStruct* prev = NULL;
    for (uint i = 0; i < numGrads; i++) {
        gradStruct* g = new gradStruct;
        g->lDelta = rows[6 * i]; g->bDelta = rows[6 * i + 1]; g->readOut = rows[6 * i + 2];
        g->gx = rows[6 * i + 3]; g->gy = rows[6 * i + 4]; g->gz = rows[6 * i + 5];
        g->next = NULL;
        if (prev) prev->next = g; else gGrads = g;
        prev = g;
    }
    timeStep = (float)kvd(kv, "timeStep", 0.01);
    stepsPerUpdate = (int)kvd(kv, "stepsPerUpdate", 1);
    numSpins = (uint)kvd(kv, "numSpins", 30000);
    gyroMagneticRatio = (float)kvd(kv, "gamma", 42576.0);
    extraAdc = (float)kvd(kv, "extraAdc", 2.1);
    intraAdc = (float)kvd(kv, "intraAdc", 2.1);
    myelinAdc = (float)kvd(kv, "myelinAdc", 0.1);
    spaceScale = (float)kvd(kv, "spaceScale", 100.0);
    permeability = (float)kvd(kv, "permeability", 0.0);
    std::string ff = kv["fiberFile"], om = kv["outm"];
    fiberFile = (char*)ff.c_str();
    outFileName = (char*)om.c_str();
    numOutputs = 6 + 4 + 1;
    gradientDataResults = new float[(size_t)numGrads * numOutputs];
    memset(gradientDataResults, 0, sizeof(float) * numGrads * numOutputs);
    psystem = &rec;
    for (uint k = 0; k < 50000000u && !computedOutput; k++) update();
    if (!computedOutput) { fprintf(stderr, "sequence did not finish\n"); return 3; }
    double tensors[5][3][3], eigenvecs[5][3][3];
    float lambdas[5][3], mds[5], fas[5], rds[5];
    for (uint c = 0; c < 5; c++) computeTensor(c, tensors, eigenvecs, lambdas, mds, fas, rds);
    FILE* f = fopen(kv["out"].c_str(), "wb");
    dump_rec(f, "calls", "f4", rec.calls.data(), rec.calls.size(), 4);
    dump_rec(f, "events", "f4", rec.events.data(), rec.events.size(), 4);
    dump_rec(f, "results", "f4", gradientDataResults, (uint64_t)numGrads * numOutputs, 4);
    dump_rec(f, "tensors", "f8", tensors, 45, 8);
    dump_rec(f, "eigenvecs", "f8", eigenvecs, 45, 8);
    dump_rec(f, "lambdas", "f4", lambdas, 15, 4);
    dump_rec(f, "md", "f4", mds, 5, 4);
    dump_rec(f, "fa", "f4", fas, 5, 4);
    dump_rec(f, "rd", "f4", rds, 5, 4);
    fclose(f);
    return 0;
}
