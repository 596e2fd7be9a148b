/*
 * dsim_serve.h -- request loop over a batch: continuous batching of
 * simulation jobs on one GPU (libdsim_gb300.so).
 *
 * No counterpart in the reference (rfdougherty/dSim runs one simulation per
 * process, dSim3/src/diffusion.cpp:1068).  A server owns a dsim_batch and a
 * worker thread.  Clients submit jobs (dsim_job_desc, initial spins, and the
 * gradients whose signals they want) at any time; the worker admits pending
 * jobs in arrival order while the batch has free spin slots and the device
 * footprint of the admitted jobs and the resident substrates stays within
 * the HBM cap, advances all admitted jobs together in quanta of whole chunks
 * (about 0.2 s of device time at the last quantum's rate, at most
 * chunk x graphChunks steps), and when a job finishes computes its signals,
 * records the time and frees its slots for the next arrivals.  Every admitted
 * job advances at the batch's step rate, so the spin capacity also bounds a
 * job's time in the batch: a few million slots keep the GPU full while jobs
 * finish quickly.  A job's result
 * does not depend on which other jobs share the batch (dsim_batch.h).
 *
 * Times are seconds since dsim_server_start on a steady clock.
 */
#ifndef DSIM_SERVE_H
#define DSIM_SERVE_H
#include <stdint.h>
#include "dsim_batch.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct dsim_server dsim_server;

/* spinCapacity / jobCapacity: the batch arena; hbmCapBytes: admission cap on
 * substrates + admitted jobs' footprint, counting, from the first job of a
 * precision form (DSIM_JOB_PRECISE / DSIM_JOB_LOCAL) on, the arena's FP64
 * fields (64 B per spin slot) and each such job's mesh FP64 triangle table
 * (128 B per triangle).  A job's host arrays are released once it is admitted. */
int dsim_server_create(uint64_t spinCapacity, uint32_t jobCapacity, uint64_t hbmCapBytes,
                       dsim_server** out);
void dsim_server_free(dsim_server* s);
/* substrates are registered before dsim_server_start */
int dsim_server_add_mesh(dsim_server* s, const dsim_mesh* m, uint32_t* substrate);
int dsim_server_add_cyl(dsim_server* s, const dsim_cyl* c, uint32_t* substrate);
int dsim_server_configure(dsim_server* s, uint32_t chunk, uint32_t occupancy, uint32_t graphChunks);
int dsim_server_start(dsim_server* s);
/* Copies the job and its inputs and returns at once.  gradScaled: nG
 * gradients (3 floats each, G[mT/m] * 1e-9 * spaceScale) sharing the job's
 * waveform.  DSIM_ETOOLARGE if the job can never fit the arena or the cap. */
int dsim_server_submit(dsim_server* s, const dsim_job_desc* job, const float* pos3,
                       const uint8_t* compartment, const uint32_t* fiber, const float* gradScaled,
                       uint32_t nG, uint32_t* ticket);
/* done = 1 when the signals are ready: out[15 g + 3 c + k] (dsim_batch_signal);
 * times = {submitted, admitted, done}; either pointer may be NULL */
int dsim_server_poll(dsim_server* s, uint32_t ticket, int* done, double* out, double times[3]);
/* block until every submitted job is done */
int dsim_server_drain(dsim_server* s);
/* stop the worker after the jobs already submitted are done */
int dsim_server_stop(dsim_server* s);
/* {jobs done, spin-steps done, busy seconds (worker advancing), largest
 *  number of jobs in flight, peak admitted HBM bytes, quanta, compactions,
 *  worker errors} */
int dsim_server_stats(dsim_server* s, double stats[8]);

#ifdef __cplusplus
}
#endif
#endif
