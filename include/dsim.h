/*
 * dsim.h -- native C-ABI of the GB300 dSim engine (libdsim_gb300.so).
 *
 * The engine runs dSim's Monte-Carlo diffusion-MRI hot path on one GB300:
 * seeded random-walk spins, collision with triangle-mesh and cylinder
 * membranes (reflection / probabilistic permeation), and phase accumulation
 * under the diffusion gradient.  All functions return 0 on success or a
 * negative status (DSIM_E*); they never abort the process.  dsim_last_error()
 * returns a message for the last failure on the calling thread.
 *
 * Coordinates are the reference's normalised units: x_norm = x_um / spaceScale,
 * box [-1, 1]^3 (rfdougherty/dSim dSim3/src/spinSystem.cpp:422-424).
 *
 * The drop-in replacements for the reference's own plugin boundary are in
 * dsim3_abi.h (dSim3/src/spinSystem.cuh) and dsim2_abi.h (dSim2/src/spinSystem.cuh).
 */
#ifndef DSIM_GB300_H
#define DSIM_GB300_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define DSIM_OK 0
#define DSIM_EINVAL (-1)
#define DSIM_ECUDA (-2)
#define DSIM_EFILE (-3)
#define DSIM_EFORMAT (-4)
#define DSIM_ENOMEM (-5)
#define DSIM_ETOOLARGE (-6)
#define DSIM_EGRID (-7)

/* status bits reported by dsim_spins_status */
#define DSIM_STATUS_SUBSEG_CAP 1u  /* a step hit the collision sub-segment cap */
#define DSIM_STATUS_BAD_CELL 2u    /* a grid list referenced a missing fiber    */
#define DSIM_STATUS_PARITY_OVERFLOW 4u /* compartment search: > 32 membranes on one line */
#define DSIM_STATUS_UNRESOLVED 8u  /* compartment search: no unambiguous line found */

typedef struct dsim_mesh dsim_mesh;
typedef struct dsim_cyl dsim_cyl;
typedef struct dsim_spins dsim_spins;

const char* dsim_last_error(void);
int dsim_version(void);
/* name (<= len bytes), SM count, global memory bytes of the current device */
int dsim_device_info(char* name, int len, int* smCount, size_t* totalMem);

/* ---- triangle-mesh substrate -------------------------------------------
 * dsim_mesh_load parses the reference's mesh fiber file (V / T / A<k> /
 * M<k> / G<k> blocks; SpinSystem::initFibers, dSim3/src/spinSystem.cpp:290-673),
 * divides vertices by spaceScale, and builds the uniform grid of numCubes^3
 * cells on the GPU with the reference's triangle/cell membership rule
 * (SpinSystem::populateCubes, spinSystem.cpp:1094-1352; the reference fixes
 * numCubes = 50).  dsim_mesh_create does the same from arrays: vertices in
 * micrometres (3 per vertex), trgls (3 vertex indices per triangle), and per
 * triangle its membrane type (0 axon, 1 myelin, 2 glia) and fiber index. */
int dsim_mesh_load(const char* path, float spaceScale, uint32_t numCubes, dsim_mesh** out);
int dsim_mesh_create(const float* vertices_um, uint32_t nVertices, const uint32_t* trgls,
                     const uint32_t* membrane, const uint32_t* fiber, uint32_t nTriangles,
                     float spaceScale, uint32_t numCubes, dsim_mesh** out);
/* info[0..7] = nVertices, nTriangles, nFibers, numCubes, grid entries,
 *              max entries in one cell, device bytes, nonempty cells */
int dsim_mesh_info(const dsim_mesh* m, uint64_t info[8]);
/* The step kernels find candidate triangles in a finer acceleration grid
 * (each triangle listed in every fine cell it touches) and
 * apply the reference grid's first-cell-with-hit rule only to the hits, which
 * gives the same results.  Built with 2.5 * numCubes cells per axis by default;
 * dsim_mesh_set_accel rebuilds it (0 = scan the reference grid directly).
 * info = {cells per axis, entries, device bytes}. */
int dsim_mesh_set_accel(dsim_mesh* m, uint32_t cellsPerAxis);
/* step kernel on the fine grid (all give the same results; default 8; other
 * values are refused): 5, 6, 7 the warp's candidate records flattened into one
 * list, lanes stepping independently (8, 6, 4 resident blocks of 128 threads
 * per SM); 8 as 6 at 5 blocks per SM (96 registers, no spills), with the
 * records that pass the plane test queued and finished 32 at a time; 9 as 6, with each lane's part of every 64-record
 * window copied into shared memory by TMA bulk copies (cp.async.bulk,
 * mbarrier completion) while the previous window is tested (8 and 9: 32-byte
 * records) */
int dsim_mesh_set_kernel(dsim_mesh* m, uint32_t variant);
/* fine-grid record size: 32 (default) holds the plane data for the exact
 * plane test; 16 holds a prefilter record only (half the bytes, one more
 * dependent load for records that pass); 64 holds everything the exact
 * triangle test reads (no dependent load) */
int dsim_mesh_set_records(dsim_mesh* m, uint32_t bytesPerRecord);
int dsim_mesh_accel_info(const dsim_mesh* m, uint64_t info[3]);
/* Compartment and fiber of every spin of `s` from its position (the
 * reference's findSpinsInFibers, dSim3/src/spinSystem.cpp:1615-1852): parity of
 * the crossings of a line out of the volume with each closed membrane,
 * innermost membrane type first; ambiguous lines (edge or vertex hits) are
 * tilted and retried 20 times, then the spin is moved to a random position in
 * [-startBoxSize, startBoxSize]^3 (draws from Philox keyed by seed).  Writes
 * the compartment and fiber (and moved positions) into s; *moved = spins
 * moved.  Needs the mesh's fine grid with 32-byte records. */
int dsim_mesh_compartments(dsim_mesh* m, dsim_spins* s, uint64_t seed, float startBoxSize, uint32_t* moved);
/* copies the CSR grid: cellStart[numCubes^3 + 1], cellTri[entries] */
int dsim_mesh_grid(const dsim_mesh* m, uint32_t* cellStart, uint32_t* cellTri);
/* copies normalised vertices[3V] and triInfo[3T] = {fiber, membrane, first vertex} */
int dsim_mesh_arrays(const dsim_mesh* m, float* vertices, uint32_t* triInfo);
void dsim_mesh_free(dsim_mesh* m);

/* ---- cylinder substrate -------------------------------------------------
 * dsim_cyl_load reads the reference's cylinder file (x y z r per line, INF
 * marks the axis; SpinSystem::initFibers(FILE*), dSim2/src/spinSystem.cpp:323-385)
 * and builds the reference's grid (build/addEntities, :135-228, 483-745).
 * fiberPos: {x, y, z, r^2} normalised with the axis coordinate 2.0. */
int dsim_cyl_load(const char* path, float spaceScale, dsim_cyl** out);
int dsim_cyl_create(const float* fiberPos4, uint32_t nFibers, float maxRadius, dsim_cyl** out);
/* geom = {numCubes, maxFibersPerCube, nFibers}; cubeLength; dense grid copies
 * (either pointer may be NULL) */
int dsim_cyl_info(const dsim_cyl* c, uint32_t geom[3], float* cubeLength, uint32_t* cubeCounter,
                  uint32_t* cubes, float* fiberPos4);
/* Fine filter grid over the reference grid, built by default: each grid cell
 * split k x k x k ways (k about twice the grid cell over the largest radius,
 * at most 16); a fine cell lists, in list order, the grid cell's entries whose
 * fiber can contain a point of it.  A spin outside every fiber tests only
 * those while its tested point stays in the cell, with results equal to the
 * full list scan.  dsim_cyl_set_fine rebuilds it with k cells per grid cell
 * edge (0 or 1: none; at most (numCubes k)^3 = 2^24 cells; call it before
 * the substrate is added to a batch).  info = {k, fine entries, bytes}. */
int dsim_cyl_set_fine(dsim_cyl* c, uint32_t k);
int dsim_cyl_fine_info(const dsim_cyl* c, uint64_t info[3]);
/* The fine lists dsim_cyl_set_fine builds, computed on the host (no device
 * call) from a reference grid: start[(numCubes k)^3 + 1] offsets and each
 * entry's position in its grid cell's list; fine cell (gx, gy, gz) is
 * (gz nk + gy) nk + gx, nk = numCubes k, inside grid cell (g / k).
 * *entries = the entry count; positions (may be NULL) holds `capacity`. */
int dsim_cyl_fine_lists(const float* fiberPos4, uint32_t nFibers, uint32_t numCubes, uint32_t maxFibersPerCube,
                        float cubeLength, const uint32_t* cubeCounter, const uint32_t* cubes, uint32_t k,
                        uint32_t* start, uint32_t* positions, uint64_t capacity, uint64_t* entries);
void dsim_cyl_free(dsim_cyl* c);

/* ---- spin state (device resident, one CUDA stream per object) ---------- */
int dsim_spins_create(uint32_t N, dsim_spins** out);
uint32_t dsim_spins_count(const dsim_spins* s);
/* mesh state: pos3 (x,y,z per spin), mag, phase, compartment, fiber */
int dsim_spins_set(dsim_spins* s, const float* pos3, const float* mag, const float* phase,
                   const uint8_t* comp, const uint16_t* fiber);
int dsim_spins_get(dsim_spins* s, float* pos3, float* mag, float* phase, uint8_t* comp,
                   uint16_t* fiber);
/* cylinder state: pos3, mag, phase, imo (0 core, 1 myelin, 2 outside), nearest fiber */
int dsim_spins_set_cyl(dsim_spins* s, const float* pos3, const float* mag, const float* phase,
                       const uint32_t* imo, const uint32_t* nearest);
int dsim_spins_get_cyl(dsim_spins* s, float* pos3, float* mag, float* phase, uint32_t* imo,
                       uint32_t* nearest);
/* per-spin collision counters {reflections or rejections, permeations} */
int dsim_spins_counts(dsim_spins* s, uint32_t* counts2N, int reset);
/* per-spin number of grid entries (candidate triangles) the step scanned,
 * accumulated by dsim_mesh_run when countCollisions has bit 2 set */
int dsim_spins_scanned(dsim_spins* s, uint32_t* scannedN, int reset);
int dsim_spins_status(dsim_spins* s, uint32_t* status, int reset);
/* Spins are reordered by fine-grid cell every `steps` steps of a mesh run
 * (default 1000, i.e. once at the start of a call of up to 1000 steps; 0 =
 * never) so that neighbouring threads read the same cell records; one step
 * kernel launch covers the steps between reorderings.  Each spin keeps its
 * identity (random stream, counters, getters). */
int dsim_spins_set_sort_interval(dsim_spins* s, uint32_t steps);
/* Global index of this object's spin 0 in the Philox counter (default 0).
 * A job split over several GPUs gives each shard the index of its first spin,
 * so the shards together draw exactly what one GPU running all spins draws. */
int dsim_spins_set_spin_base(dsim_spins* s, uint32_t base);
/* bytes of device memory held by the object */
uint64_t dsim_spins_bytes(const dsim_spins* s);
void dsim_spins_free(dsim_spins* s);

/* ---- stepping ------------------------------------------------------------
 * countCollisions: bit 0 accumulates per-spin {reflections, permeations},
 * bit 1 (value 2) accumulates the grid entries each spin scanned.
 * One launch advances every spin `iterations` steps with state held in
 * registers.  g = scaled gradient (G[mT/m] * 1e-9 * spaceScale,
 * SpinSystem::updateSpins dSim3/src/spinSystem.cpp:1931) used for every step,
 * unless gradPerStep (host, 3 floats per step) is given.  Draws come from
 * Philox4x32-10 with key = seed and counter = (spin, step0 + step, stream),
 * or, when replayDraws (host, [iterations][N][4] = n.x, n.y, n.z, u) is given,
 * from that stream (replay mode). */
typedef struct {
    float stdDevs[4];       /* per compartment, normalised (sqrt(2 ADC dt)/spaceScale) */
    float T2[4];            /* ms */
    float permeability;     /* probability per membrane hit */
    uint32_t reflectionType;/* 1 mirror, 0 back to the segment start */
    float spinRadius;       /* clamp margin, 0.005 in the reference */
    float deltaTime;        /* ms */
    float phaseConstant;    /* 2 pi gamma dt */
    uint32_t maxSubsegments;/* collision sub-segments per step before flagging (0 = 4096) */
} dsim_mesh_params;

int dsim_mesh_run(dsim_mesh* m, dsim_spins* s, const dsim_mesh_params* p, const float g[3],
                  const float* gradPerStep, uint32_t iterations, uint64_t seed, uint64_t step0,
                  const float* replayDraws, int countCollisions);

typedef struct {
    float intraAdc, extraAdc, myelinAdc; /* um^2/ms */
    float spaceScale;
    float T2fiber, T2myelin, T2outside;  /* ms */
    float permeability;
    float innerRadiusProportion;
    float spinRadius;
    float deltaTime;
    float phaseConstant;
} dsim_cyl_params;

int dsim_cyl_run(dsim_cyl* c, dsim_spins* s, const dsim_cyl_params* p, const float g[3],
                 const float* gradPerStep, uint32_t iterations, uint64_t seed, uint64_t step0,
                 const float* replayDraws, int countCollisions);

/* Ensemble signal in FP64: out[3c + 0..2] = {sum m cos(phi), sum m sin(phi), n}
 * for c = 0 (all spins) and c = 1 + compartment (mesh) / 1 + imo (cylinders).
 * region > 0 keeps spins with |x|,|y|,|z| < region (dSim2 uses 0.8).
 * A spin whose compartment index is above 3 is counted in c = 0 only, so
 * out[2] minus the four compartment counts is the number of such spins (the
 * reference's arrays hold four compartments and would overrun). */
int dsim_signal(dsim_spins* s, double region, double out[15]);

/* dsim_signal over the reference's own device spin arrays, allocating
 * nothing (no counterpart in the reference, whose getMrSignal copies every
 * spin to the host: dSim3/src/spinSystem.cpp:1452-1500,
 * dSim2/src/spinSystem.cpp:944-978).  For callers that cannot allocate device
 * memory when they need the signal.
 *   layout DSIM_SIGNAL_DSIM3: pos = float3[N], spinRecords = spinData[N]
 *          (12 B: mag, phase, compartment byte, pad, fiber u16)
 *   layout DSIM_SIGNAL_DSIM2: pos = float4[N] {x, y, z, phase},
 *          spinRecords = uint4 seeds[N] or NULL; mag = 1.  Word 2 holds
 *          imo + 1, or 0 as the reference's assignSeeds leaves it, when
 *          word 3 (nearest fiber, UINT_MAX outside) gives core or outside
 * out: DEVICE pointer to 15 doubles, same meaning as dsim_signal; written
 * asynchronously on `stream` (a cudaStream_t; NULL = legacy default stream).
 * Scratch is a fixed array inside the library (983,040 bytes): N above
 * 16,777,216 returns DSIM_ETOOLARGE.  Nothing must start at zero.  Every
 * call looks up the scratch address (allocating nothing); the first call on a
 * device loads the library's module there, so make it before any stream
 * capture.  Calls that may overlap in time race on the one scratch array:
 * serialise them (e.g. issue them on one stream). */
#define DSIM_SIGNAL_DSIM3 1
#define DSIM_SIGNAL_DSIM2 2
int dsim_signal_noalloc(const float* pos, const void* spinRecords, uint32_t N, int layout,
                        double region, double* out, void* stream);

/* The draws the step kernels use: for spins [spin0, spin0 + n) at global
 * step `step` with key `seed` and counter word `stream`, writes the Philox
 * words (raw, 4 per spin, may be NULL) and (n.x, n.y, n.z, u) (draws4). */
int dsim_rng_draws(uint64_t seed, uint32_t spin0, uint64_t step, uint32_t stream, uint32_t n,
                   uint32_t* raw, float* draws4);

/* number of kernels dsim_mesh_run / dsim_cyl_run launched for this object
 * (step kernels, spin sorts, reorderings) since the last reset */
int dsim_spins_launches(dsim_spins* s, uint64_t* n, int reset);

/* stream control and device timing on the object's stream */
int dsim_sync(dsim_spins* s);
int dsim_timer_start(dsim_spins* s);
int dsim_timer_stop(dsim_spins* s, float* ms);
/* writes `bytes` to a scratch buffer on the object's stream (cache flush) */
int dsim_flush_l2(dsim_spins* s, size_t bytes);

#ifdef __cplusplus
}
#endif
#endif
