/*
 * dsim_sim.h -- the reference's simulate call around the GPU path
 * (libdsim_gb300.so): sim.cfg / .grads / fiber-file inputs, the PGSE
 * sequencer, the signal per gradient, the diffusion-tensor fit and the
 * MATLAB results file.
 *
 * Reference: dSim3/src/diffusion.cpp (config 148-202, sequencer update()
 * 522-737, computeTensor 286-511, results writer 666-728) and
 * dSim2/src/diffusion.cpp (config 1095-1144, update() 183-287, results header
 * 1756-1770).  Both config dialects are read (dSim3: sim.timeStep,
 * fibers.fiberFile; dSim2: sim.timestep, fibers.file, permeability given as
 * log10).  A mesh fiber file (V/T/A/M/G blocks) selects the dSim3 mesh
 * path, a cylinder file (x y z r lines) the dSim2 cylinder path.
 */
#ifndef DSIM_SIM_H
#define DSIM_SIM_H
#include <stdint.h>
#include "dsim.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int dialect;               /* 3: dSim3 keys, 2: dSim2 keys */
    uint32_t stepsPerUpdate;
    int useGpu, useDisplay, writeOut;
    uint32_t numSpins;
    float gamma;               /* gyromagnetic ratio / 2 pi, kHz/T */
    float timeStep;            /* ms */
    float extraAdc, intraAdc, myelinAdc;   /* um^2/ms */
    float extraT2, intraT2, myelinT2;      /* ms */
    float spaceScale;          /* um per normalised unit */
    float startBox;            /* spins start in [-startBox, startBox]^3 (dSim3) */
    float permeability;        /* probability per hit (dSim2's log10 value converted) */
    float innerRadiusFraction; /* dSim2 fibers.innerRadiusFraction */
    char gradsFile[512], gradsStr[512], outFile[512], fiberFile[512];
    /* dSim2 fibers.radiusMean, fibers.spacingMean, fibers.crossFraction (its
     * fiber generator's parameters, written in its results header) */
    float fiberRadius, fiberSpace, crossFraction;
} dsim_config;

/* libconfig subset (groups, scalars, strings, booleans, comments); relative
 * file names are kept as written.  Missing keys keep the reference's
 * defaults. */
int dsim_config_load(const char* path, dsim_config* out);
/* gradient rows {delta, Delta, readout (ms), Gx, Gy, Gz (mT/m)}: numbers are
 * read six at a time as the reference's fscanf("%g %g %g %g %g %g") loop
 * does; a trailing incomplete row is dropped.  rows may be NULL (count only). */
int dsim_grads_parse_file(const char* path, float* rows, uint32_t cap, uint32_t* n);
int dsim_grads_parse_string(const char* text, float* rows, uint32_t cap, uint32_t* n);
/* The sequencer's gradient for every step of one run (update() of
 * dSim3/src/diffusion.cpp:553-625): per-update counts round(delta /
 * (timeStep * stepsPerUpdate)) etc., the gradient switched at the same update
 * indices, the signal read after nUpdates * stepsPerUpdate steps.
 * gradPerStep: 3 floats per step in mT/m (may be NULL); *nSteps = steps.
 * DSIM_EINVAL for a row whose readout rounds to zero updates: update() never
 * reaches its signal read for such a row (dsim_simulate reports NaN). */
int dsim_pgse_schedule(const float row[6], float timeStep, uint32_t stepsPerUpdate, float* gradPerStep,
                       uint32_t cap, uint32_t* nSteps);
/* Diffusion tensor from the signals of nG gradient rows (computeTensor,
 * dSim3/src/diffusion.cpp:286-511): log-signal ADC per non-zero gradient,
 * least-squares tensor, eigen-decomposition (eigenvalues ascending, vectors in
 * columns), mean, fractional and radial diffusivity. */
int dsim_tensor_fit(const float* rows, const double* signal, uint32_t nG, double tensor[9], double eigvecs[9],
                    float eigvals[3], float* md, float* fa, float* rd);

/* Appends the reference's results block for one simulation to outFile.
 * dSim3 dialect (dSim3/src/diffusion.cpp:666-728): the input parameters, the
 * tensor fits of the total signal and of compartments 0-2 as indices 1-4 (the
 * reference's indexing), then every row with its signals.  dSim2 dialect
 * (dSim2/src/diffusion.cpp:1756-1770, 232-276): the header, one block per row
 * and the stepsPerSec / totalTime timing from `seconds`.  rows [nG][6],
 * signals [nG][5] as dsim_simulate returns them.  dSim3: like the reference,
 * the signals are rounded to float before they are fitted and printed, and a
 * row whose signal the sequencer never reads (NaN from dsim_simulate) holds 0,
 * as in the reference's zeroed results table.  dSim2: the total signal is
 * printed as the double it is, and a row never read gets no signal line. */
int dsim_write_results(const char* outFile, const dsim_config* cfg, const float* rows, const double* signals,
                       uint32_t nG, double seconds);

#define DSIM_SIM_SHARED_WALK 1u  /* one walk per (delta, Delta, readout) group, all its gradients from moments */
#define DSIM_SIM_WRITE_OUT 2u    /* append the results file named by sim.outFile (if writeOut) */

/* Runs the simulation a config describes on the GPU: for every gradient row
 * the spins are reset (positions from Philox keyed by seed, compartments by
 * ray parity or the nearest-cylinder search) and walked through the
 * sequencer's schedule.  signals[5 g + c]: c = 0 total, 1 + compartment
 * (dSim2: spins within +-0.8, as its getMrSignal).  seconds = device time. */
int dsim_simulate(const char* cfgPath, uint64_t seed, uint32_t flags, double* signals, uint32_t cap,
                  uint32_t* nG, double* seconds);

#ifdef __cplusplus
}
#endif
#endif
