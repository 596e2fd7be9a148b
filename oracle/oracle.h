/*
 * oracle.h -- CPU restatement of dSim's Monte-Carlo hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU engine
 * in dsim_gb300/: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it.  The product path never calls into it.
 *
 * Every function restates one function of the reference's CPU code
 * (rfdougherty/dSim) with the same floating-point expression order, so that
 * compiled with -ffp-contract=off it reproduces the reference bit for bit:
 *   dSim3 (triangle meshes):   dSim3/src/spinKernelCpu.cpp, dSim3/src/spinSystem.cpp
 *   dSim2 (cylinders):         dSim2/src/spinKernelCpu.cpp, dSim2/src/spinSystem.cpp
 * Parity of this restatement is pinned against the reference's own CPU code,
 * compiled from its sources by oracle/build_ref.py, through the fixtures in
 * tests/golden/ (generator: tests/golden/make_golden.py).
 *
 * Array conventions (identical to the reference's host arrays):
 *   pos      float[3N]   x,y,z per spin (normalised units, box [-1,1]^3)
 *   seed     uint32[2N]  MWC state per spin (dSim3) / uint32[4N] (dSim2)
 *   mag,phase float[N]   spinData.signalMagnitude / signalPhase
 *   comp     uint8[N]    spinData.compartmentType
 *   fiber    uint16[N]   spinData.insideFiber
 *   draws    float[iters][N][4]  replay stream (n.x, n.y, n.z, u); NULL = MWC
 *   counts   uint32[2N]  per spin: reflections, permeations (accumulated)
 */
#ifndef DSIM_ORACLE_H
#define DSIM_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* ---- Philox4x32-10 (Salmon et al., SC'11), reference for the GPU generator */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* ---- dSim3 mesh substrate (dSim3/src/spinSystem.cpp:290-673) -------------
 * counts[0..6] = nVertices, nTriangles, nFibers, nAxon, nMyelin, nGlia,
 *                maxTrianglesOnSurface.  Returns 0, or -1 (cannot open),
 *                -2 (axon/myelin membrane count mismatch, spinSystem.cpp:593). */
int or3_mesh_count(const char* path, uint32_t counts[7]);
/* fills vertices[3V] (divided by spaceScale), trgls[3T], triInfo[3T],
 * helpers[12T], maxabs[3] = m_xmax, m_ymax, m_zmax */
int or3_mesh_fill(const char* path, float spaceScale, const uint32_t counts[7],
                  float* vertices, uint32_t* trgls, uint32_t* triInfo,
                  float* helpers, float maxabs[3]);

/* ---- dSim3 rectangular grid (spinSystem.cpp:1094-1352) ------------------- */
/* pass 1: cubeCounter[n^3] and returns maxTrianglesPerCube */
uint32_t or3_populate_count(uint32_t nT, const float* vertices, const uint32_t* trgls,
                            uint32_t numCubes, uint32_t* cubeCounter);
/* pass 2: dense trianglesInCubes[n^3 * maxTPC] (cubeCounter rewritten) */
void or3_populate_fill(uint32_t nT, const float* vertices, const uint32_t* trgls,
                       uint32_t numCubes, uint32_t maxTPC, uint32_t* cubeCounter,
                       uint32_t* trianglesInCubes);

/* ---- dSim3 step: updateSpins -> cpuIntegrateSystem -> cpuIntegrate ------- */
typedef struct {
    float stdDevs[4];      /* m_hStdDevs, spinSystem.cpp:52-56 */
    float T2[4];           /* m_hT2Values, spinSystem.cpp:47-51 */
    float permeability;
    uint32_t reflectionType;
    float spinRadius;      /* 0.005 (spinSystem.cpp:62) */
    float deltaTime;
    uint32_t numCubes;
    uint32_t maxTrianglesPerCube;
    float cubeLength;
    uint32_t maxSubsegments; /* safety cap on the sub-segment loop (0 = 1<<20) */
} or3_params;

/* returns the number of spins that hit maxSubsegments (0 in normal use) */
uint32_t or3_integrate(const or3_params* p, uint32_t N, float* pos, uint32_t* seed,
                       float* mag, float* phase, uint8_t* comp, uint16_t* fiber,
                       const float* vertices, const float* helpers,
                       const uint32_t* triInfo, const uint32_t* cubeCounter,
                       const uint32_t* trianglesInCubes, float gx, float gy, float gz,
                       float phaseConstant, uint32_t iterations, const float* draws,
                       float* drawsOut, uint32_t* counts);

/* or3_integrate with the spin loop over nthreads OpenMP threads (MWC draws) */
uint32_t or3_integrate_mt(const or3_params* p, uint32_t N, float* pos, uint32_t* seed,
                          float* mag, float* phase, uint8_t* comp, uint16_t* fiber,
                          const float* vertices, const float* helpers,
                          const uint32_t* triInfo, const uint32_t* cubeCounter,
                          const uint32_t* trianglesInCubes, float gx, float gy, float gz,
                          float phaseConstant, uint32_t iterations, int nthreads);

/* FP64 restatement of the same step (precision oracle): same algorithm,
 * doubles throughout, triangle helpers recomputed in double from vertices
 * (double[3V]); draws are the same float stream.  Grid as in the FP32 path. */
uint32_t or3_integrate_f64(const or3_params* p, uint32_t N, double* pos, double* mag,
                           double* phase, uint8_t* comp, uint16_t* fiber,
                           uint32_t nT, const double* vertices, const uint32_t* trgls,
                           const uint32_t* triInfo, const uint32_t* cubeCounter,
                           const uint32_t* trianglesInCubes, const double* gradPerStep,
                           double phaseConstant, uint32_t iterations, const float* draws,
                           uint32_t* counts);

/* the FP64 walk recording gradient moments M_k = sum_t w_k(t) pos(t) for
 * nWaves waveforms (moments[N][nWaves][3]); OpenMP over spins */
uint32_t or3_integrate_f64_moments(const or3_params* p, uint32_t N, double* pos, double* mag,
                                   uint8_t* comp, uint16_t* fiber, uint32_t nT,
                                   const double* vertices, const uint32_t* trgls,
                                   const uint32_t* triInfo, const uint32_t* cubeCounter,
                                   const uint32_t* trianglesInCubes, uint32_t nWaves,
                                   const double* waves, uint32_t iterations, const float* draws,
                                   double* moments, uint32_t* counts, int nthreads);

/* The reference's walk for nG gradient runs at once.  The walk (positions,
 * compartments, magnitudes) does not depend on the gradient, so one walk
 * with the reference's own MWC draws (seed[2N], or replay draws) serves every
 * run: after each step, for run k, phases[i*nG + k] += (gx*x + gy*y + gz*z)*pc
 * with g = wave[t] * grads[k] in float -- the reference's phase update
 * (spinKernelCpu.cpp:490) for the gradient the sequencer passes at step t
 * (wave 1, 0, -1 for PGSE: diffusion.cpp:553-625).  OpenMP over spins (each
 * spin's MWC stream is its own, so the result does not depend on nthreads). */
uint32_t or3_integrate_multi(const or3_params* p, uint32_t N, float* pos, uint32_t* seed,
                             float* mag, uint8_t* comp, uint16_t* fiber,
                             const float* vertices, const float* helpers,
                             const uint32_t* triInfo, const uint32_t* cubeCounter,
                             const uint32_t* trianglesInCubes, uint32_t nG, const float* grads,
                             const float* wave, float phaseConstant, uint32_t iterations,
                             const float* draws, float* phases, uint32_t* counts, int nthreads);

/* getMrSignal(double[]) spinSystem.cpp:1452-1500: out[0]=total, out[1+c]=c */
void or3_signal(uint32_t N, const float* mag, const float* phase, const uint8_t* comp,
                double out[5]);

/* ---- dSim2 cylinders ------------------------------------------------------ */
/* initFibers(FILE*) dSim2/src/spinSystem.cpp:323-385.  First call with
 * fiberPos NULL to count; returns number of fibers kept, maxR in *maxR */
int or2_load_fibers(const char* path, float spaceScale, float* fiberPos, float* maxR);
/* build()+addEntities() dSim2/src/spinSystem.cpp:135-228, 483-745.
 * geom[0]=numCubes, geom[1]=maxFibersPerCube; cubeLength in *cubeLength.
 * With cubeCounter NULL only geometry is computed.  Returns 0 or -1 if a
 * cell overflows maxFibersPerCube (the reference's build() then fails). */
int or2_build_grid(uint32_t nF, const float* fiberPos, float maxR, uint32_t geom[2],
                   float* cubeLength, uint32_t* cubeCounter, uint32_t* cubes);
/* findNearestFiber dSim2/src/spinSystem.cpp:1223-1311 for spins [0,N) */
void or2_find_nearest(uint32_t N, const float* pos4, const float* fiberPos,
                      uint32_t numCubes, float cubeLength, uint32_t maxFPC,
                      const uint32_t* cubeCounter, const uint32_t* cubes,
                      float innerRadiusProportion, uint32_t* nearest, uint32_t* imo);

typedef struct {
    float intraAdcScaled, extraAdcScaled, myelinAdcScaled; /* ADC/spaceScale^2 */
    float T2fiber, T2myelin, T2outside;
    float permeability;
    float innerRadiusProportion;
    float spinRadius;
    float deltaTime;
    uint32_t numCubes, maxFibersPerCube;
    float cubeLength;
} or2_params;

/* cpuIntegrateSystem dSim2/src/spinKernelCpu.cpp:2-20 / cpuIntegrate 312-641
 * pos4 float[4N], seed4 uint32[4N], params float[5N] {mag, phase, nearest, imo, -} */
void or2_integrate(const or2_params* p, uint32_t N, float* pos4, uint32_t* seed4,
                   float* params5, const float* fiberPos, const uint32_t* cubeCounter,
                   const uint32_t* cubes, float gx, float gy, float gz,
                   float phaseConstant, uint32_t iterations, const float* draws,
                   float* drawsOut, uint32_t* counts);

/* or2_integrate for nG gradient runs at once (see or3_integrate_multi):
 * one walk with the reference's MWC draws (seed4 words 0-1) or replay draws;
 * phases[i*nG + k] += (gx*x + gy*y + gz*z)*pc with g = wave[t] * grads[k]
 * (dSim2/src/spinKernelCpu.cpp:636).  OpenMP over spins. */
void or2_integrate_multi(const or2_params* p, uint32_t N, float* pos4, uint32_t* seed4,
                         float* params5, const float* fiberPos, const uint32_t* cubeCounter,
                         const uint32_t* cubes, uint32_t nG, const float* grads, const float* wave,
                         float phaseConstant, uint32_t iterations, const float* draws,
                         float* phases, uint32_t* counts, int nthreads);

/* FP64 precision oracle for cylinders: the same walk with every
 * position-dependent quantity in double, on replay draws (float[iters][N][4]),
 * one walk for nG gradient runs (phases[i*nG + k] in double).  pos3, mag,
 * imo, nearest are updated in place.  OpenMP over spins. */
void or2_integrate_f64_multi(const or2_params* p, uint32_t N, double* pos3, double* mag, uint32_t* imo,
                             uint32_t* nearest, const float* fiberPos, const uint32_t* cubeCounter,
                             const uint32_t* cubes, uint32_t nG, const double* grads, const double* wave,
                             double phaseConstant, uint32_t iterations, const float* draws, double* phases,
                             int nthreads);

/* getMrSignal() dSim2/src/spinSystem.cpp:944-978 (spins inside +-0.8 only) */
double or2_signal(uint32_t N, const float* pos4, const float* params5);

/* MWC + Box-Muller as in spinKernelCpu.cpp:41-63 (both trees): one step of
 * draws for one spin; seed is updated.  Exposed so tests can regenerate. */
void or_myrandn(uint32_t seed[2], float out[4]);

#ifdef __cplusplus
}
#endif
#endif
