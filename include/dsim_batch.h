/*
 * dsim_batch.h -- many simulation jobs in one step launch (libdsim_gb300.so).
 *
 * No counterpart in the reference: rfdougherty/dSim runs one substrate and
 * one gradient per walk, one walk after another (dSim3/src/diffusion.cpp:553-625
 * resets the spins for every gradient).  A batch holds the spins of many jobs
 * (each with its own substrate, step count, time step, diffusivities, T2,
 * permeability, waveform and seed) packed in one device array with a per-spin
 * job index, and advances all of them with one step launch per chunk of steps.
 *
 * Per spin the batch keeps the gradient moment M = sum_t w(t) pos(t) (w: the
 * job's waveform, pos: normalised position after step t) with compensated
 * (Kahan) FP32 summation (FP64 in the precision form), instead of one phase.  Every gradient G that shares
 * the waveform then has phase phi = phaseConstant * (gradScaled(G) . M),
 * evaluated in FP64 at readout, so one walk serves all directions and
 * magnitudes of a gradient table.  The mesh step rules, random draws and
 * positions are those of dsim_mesh_run (a job alone in a batch reproduces
 * dsim_mesh_run's positions bit for bit); cylinder jobs follow dsim_cyl_run.
 *
 * All functions return 0 or a negative DSIM_E* status (dsim.h); a batch is
 * used from one host thread at a time.
 */
#ifndef DSIM_BATCH_H
#define DSIM_BATCH_H
#include <stddef.h>
#include <stdint.h>
#include "dsim.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct dsim_batch dsim_batch;

#define DSIM_WAVE_PGSE 0  /* +1 for steps [0, nd), -1 for [nD, nD + nd), else 0 */
#define DSIM_WAVE_OGSE 1  /* cos(2 pi f t) on [0, nd), -cos(2 pi f (t - Delta)) on [nD, nD + nd) */
#define DSIM_WAVE_TABLE 2 /* explicit w(t), one value per step */

typedef struct {
    uint32_t substrate;    /* index from dsim_batch_add_mesh / dsim_batch_add_cyl */
    uint32_t nSpins;
    uint32_t steps;
    float deltaTime;       /* ms */
    float stepSd[4];       /* normalised step sigma per compartment: mesh 0 extra,
                              1 intra, 2 myelin, 3 glia; cylinders 0 core, 1 myelin, 2 outside */
    float T2[4];           /* ms per compartment; <= 0: no decay */
    float permeability;
    uint32_t reflectionType;       /* mesh: 1 mirror reflection, 0 back to the segment start */
    float spinRadius;              /* positions clamp to +-(1 - spinRadius) */
    float innerRadiusProportion;   /* cylinders: myelin inner radius / outer radius */
    float phaseConstant;           /* 2 pi gamma dt, as SpinSystem::updateSpins */
    uint32_t waveform;             /* DSIM_WAVE_* */
    float delta, Delta;            /* ms (PGSE, OGSE); step counts nd = round(delta/dt) */
    float frequency;               /* Hz (OGSE) */
    const float* table;            /* DSIM_WAVE_TABLE: `steps` values (host) */
    uint64_t seed;                 /* Philox key; counter = (spin, step, 0) */
    uint32_t flags;                /* DSIM_JOB_PRECISE or DSIM_JOB_LOCAL (mesh or cylinder jobs) */
    uint32_t reserved;
} dsim_job_desc;

/* Precision form: the job's step is the reference algorithm evaluated in FP64
 * -- positions, sub-segments, triangle tests on FP64 triangle helpers (the
 * formulas of dSim3/src/spinSystem.cpp:612-648 in double), reflections, the
 * clamp, T2 decay and the gradient moments -- on the same draws as the plain
 * form; FP32 only prunes fine-grid records whose plane lies clearly off the
 * sub-segment.  For a cylinder job it is the dSim2 step
 * (dSim2/src/spinKernelCpu.cpp:312-641) with positions, distances to the
 * fibers, the clamp, T2 decay and moments in FP64 (the fiber records and the
 * other parameters are the job's float values).  Positions and magnitudes
 * persist in FP64 (dsim_batch_get_precise); dsim_batch_get returns them
 * rounded to float. */
#define DSIM_JOB_PRECISE 1u
/* Cell-local form: the plain FP32 step with every position held as an FP32
 * offset from a lattice origin (a multiple of 1/16 in normalised units), so
 * positions round about 16x finer than absolute FP32 coordinates; the
 * intersections whose FP32 outcome lies within the FP32 error band of a
 * decision boundary (crossing parameter near 0 or 1, a barycentric coordinate
 * within 1e-5 of an edge) are decided again in FP64 on the FP64 triangle
 * helpers; moments are Kahan-compensated FP32.  For a cylinder job the
 * distances to the fibers are formed in the local frame, and a membrane
 * decision whose FP32 distance lies within its error band of inR r^2 or r^2
 * is taken from the FP64 distance at the exact position, as the FP64 form
 * takes it there (grid lookups use the position rounded to float).
 * dsim_batch_precision_counts then reports distance tests and FP64
 * decisions.  Exclusive with DSIM_JOB_PRECISE.  dsim_batch_get_precise
 * returns origin + offset. */
#define DSIM_JOB_LOCAL 2u

/* spinCapacity: packed spin slots (each job is padded to a multiple of 32) */
int dsim_batch_create(uint64_t spinCapacity, uint32_t jobCapacity, dsim_batch** out);
void dsim_batch_free(dsim_batch* b);
/* substrates are shared with the batch (keep them alive while it runs); the
 * mesh needs its fine grid (dsim_mesh_set_accel > 0, the default) */
int dsim_batch_add_mesh(dsim_batch* b, const dsim_mesh* m, uint32_t* substrate);
int dsim_batch_add_cyl(dsim_batch* b, const dsim_cyl* c, uint32_t* substrate);
/* Adds a job: initial state from host arrays (pos3 normalised; compartment:
 * mesh compartment 0..3 or cylinder region imo 0..2; fiber: mesh fiber index
 * or nearest cylinder, 0xFFFFFFFF none).  The job's step 0 runs in the next
 * chunk.  DSIM_ENOMEM when spin or job capacity is exhausted. */
int dsim_batch_submit(dsim_batch* b, const dsim_job_desc* job, const float* pos3,
                      const uint8_t* compartment, const uint32_t* fiber, uint32_t* jobId);
/* chunk: steps between spin sorts (default 20); occupancy: 4 (default), 5, 6 or 8
 * resident blocks per SM for the step kernel; graphChunks: chunks captured in
 * one CUDA graph launch (0 = plain launches, default 8) */
int dsim_batch_configure(dsim_batch* b, uint32_t chunk, uint32_t occupancy, uint32_t graphChunks);
/* block size of the plain step kernels: 64, 128 (default) or 256 threads, at
 * the register budget of the configured occupancy (the other forms' kernels
 * run 128-thread blocks); dsim_batch_autotune sets it too */
int dsim_batch_set_block(dsim_batch* b, uint32_t threads);
int dsim_batch_block(const dsim_batch* b, uint32_t* threads);
/* advance every unfinished job by `steps` steps (rounded up to whole chunks) */
int dsim_batch_advance(dsim_batch* b, uint32_t steps);
/* advance until every job has finished */
int dsim_batch_run(dsim_batch* b);
/* steps done and total for a job; *done = 1 when finished */
int dsim_batch_job_status(dsim_batch* b, uint32_t jobId, uint32_t* stepsDone, int* done);
/* FP64 signal of a job for nG gradients sharing its waveform: gradScaled =
 * G[mT/m] * 1e-9 * spaceScale (3 floats per gradient); out[15 g + 3 c + k] as
 * dsim_signal (c = 0 all, 1 + compartment).  Synchronous. */
int dsim_batch_signal(dsim_batch* b, uint32_t jobId, const float* gradScaled, uint32_t nG,
                      double* out);
/* dsim_batch_signal over the spins with |x|, |y|, |z| < region only (region 0:
 * every spin).  dSim2's getMrSignal reads the box +-0.8
 * (dSim2/src/spinSystem.cpp:944-978); the simulate call passes 0.8 for
 * cylinder configurations. */
int dsim_batch_signal_region(dsim_batch* b, uint32_t jobId, const float* gradScaled, uint32_t nG,
                             double region, double* out);
/* a job's spins in spin order: pos3, mag, moments (M and its compensation,
 * 6 per spin), compartment, fiber (any pointer may be NULL).  Synchronous. */
int dsim_batch_get(dsim_batch* b, uint32_t jobId, float* pos3, float* mag, float* moments6,
                   uint8_t* compartment, uint32_t* fiber);
/* per-job {reflections or rejections, permeations} and status bits */
int dsim_batch_counts(dsim_batch* b, uint32_t jobId, uint64_t counts[2]);
/* precision and cell-local forms: {fine-grid records examined, FP64 triangle
 * tests}; cell-local cylinder jobs: {distance tests, FP64 decisions} */
int dsim_batch_precision_counts(dsim_batch* b, uint32_t jobId, uint64_t out[2]);
/* precision and cell-local forms: FP64 positions (3 per spin) and magnitudes
 * in spin order; DSIM_EINVAL for a plain job.  Synchronous. */
int dsim_batch_get_precise(dsim_batch* b, uint32_t jobId, double* pos3, double* mag);
uint32_t dsim_batch_status(dsim_batch* b);
/* drop finished jobs whose results were read and repack the others */
int dsim_batch_retire(dsim_batch* b, uint32_t jobId);
int dsim_batch_compact(dsim_batch* b);
/* Autotuner: runs the current jobs from a snapshot of the
 * spin state for every candidate -- step-kernel occupancy {4, 5, 6, 8} x chunk
 * {20, 40, 100, 200, 500, 1000} x fine-grid cells per reference-cell edge
 * {1, 1.5, 2, 2.5}; every candidate runs the same max(trialSteps, 1000) steps,
 * so longer chunks are not favoured by jobs finishing inside the trial; then,
 * at the best of those, the plain step kernels' block size {64, 128, 256}
 * (left set; dsim_batch_block reads it)
 * (every mesh substrate's fine grid is rebuilt; meshes must not be in use
 * elsewhere meanwhile) -- restores the snapshot and keeps the fastest.
 * best = {occupancy, chunk, 2 x fine cells per reference cell edge (0: no
 * mesh)}, bestMs = its time per trialSteps steps. */
int dsim_batch_autotune(dsim_batch* b, uint32_t trialSteps, uint32_t best[3], float* bestMs);
/* {packed spins, jobs, jobs running, device bytes, kernels launched, graph launches} */
int dsim_batch_info(dsim_batch* b, uint64_t info[6]);
/* wait for everything queued on the batch's stream */
int dsim_batch_sync(dsim_batch* b);

#ifdef __cplusplus
}
#endif
#endif
