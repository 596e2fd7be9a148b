// engine.h -- internal interfaces shared by the engine's translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "common.cuh"

struct dsim_mesh;
struct dsim_cyl;

namespace dsim {

enum Layout : int { kLayoutSoA = 0, kLayoutAoS = 1 };
enum Rng : int { kRngPhilox = 0, kRngReplay = 1, kRngPhiloxPerSpinKey = 2 };

// per-triangle FP64 helpers of the precision form: unit normal, first vertex,
// u = p3 - p1, v = p2 - p1, u.v, u.u, v.v, evaluated in double from the FP32
// vertices with the formulas of dSim3/src/spinSystem.cpp:612-648
struct __align__(16) Tri64 {
    double nx, ny, nz, p1x, p1y, p1z, ux, uy, uz, vx, vy, vz, uv, uu, vv, pad;
};

// device view of a mesh substrate (CSR cell lists over per-triangle records)
struct MeshDev {
    const uint32_t* cell_start;  // ncells + 1
    const uint32_t* cell_tri;    // triangle index per entry, ascending in a cell
    const TriPlane* plane;       // per triangle
    const TriBary* bary;         // per triangle
    const Tri64* tri64;          // per triangle, precision form only (else null)
    const uint4* tri_cells;      // per triangle: its reference cells (up to 4; else null)
    uint32_t n;                  // cells per axis
    float L;                     // cell edge, normalised units (2 / n)
};

// device view of spin state.  SoA: x,y,z,mag,phase float[N], meta uint32[N]
// (compartment | fiber << 8).  AoS (reference arrays): x = float3 positions,
// meta = spinData records (12 B); y, z, mag, phase unused.
struct SpinsDev {
    float *x, *y, *z, *mag, *phase;
    uint32_t* meta;
    uint32_t* seed;  // per-spin Philox key (2 words) for kRngPhiloxPerSpinKey
    uint32_t N;
};

struct MeshStepArgs {
    float sd[4];          // per-compartment step standard deviation (normalised)
    float T2[4];          // per-compartment T2 (ms)
    float perm;           // permeation probability per hit
    uint32_t reflType;    // 1 mirror reflection, 0 return to the segment start
    float clampHi, clampLo;  // 1 - spinRadius, -1 + spinRadius
    float dt, pc;         // time step (ms), phase constant 2*pi*gamma*dt
    float gx, gy, gz;     // scaled gradient, constant over the call
    const float4* grad;   // or one scaled gradient per iteration
    uint32_t iterations;
    uint32_t key0, key1;  // Philox key (kRngPhilox)
    uint64_t step0;       // global index of the first step
    uint32_t stream;      // Philox counter word 3
    const float4* draws;  // replay stream [iterations][N] (kRngReplay)
    uint32_t maxSub;      // cap on collision sub-segments per step
    uint32_t* status;     // device status word (StatusBits)
    uint32_t* counts;     // [2N] reflections, permeations (or null)
    uint32_t* tested;     // [N] grid entries scanned (or null)
    const uint32_t* spinKeys;  // per-spin Philox keys [2N] by id (kRngPhiloxPerSpinKey, fast path)
    uint32_t spinBase;    // added to the spin index in the Philox counter (replica shards)
};

// ---- accel.cu -------------------------------------------------------------
// Fine acceleration grid: every triangle is listed in each fine cell it
// touches (separating-axis test against the cell widened by kAccelEps); cells
// are stored in Morton order.  Per entry a 16-byte plane record {n.x, n.y, n.z, n.p1} for a
// conservative plane-crossing prefilter, and the triangle index beside it.
static constexpr float kAccelEps = 1e-5f;
struct __align__(16) AccelRec {
    float4 q;
};
// 32-byte record: the plane record and {p1.x, p1.y, p1.z, t} in one sector,
// so the exact plane test needs no dependent load
struct __align__(32) AccelRecWide {
    float4 q, pt;
};
// 64-byte record: everything the exact test reads, so a record is decided
// with no dependent load: {n, vv} {p1, t} {u, v.x} {v.y, v.z, uv, uu}
struct __align__(16) AccelRecFull {
    float4 a, b, c, d;
};
struct AccelDev {
    const uint32_t* start;  // Morton key -> first record (keys + 1 entries)
    const AccelRec* rec;    // 16-byte records (wide == 0)
    const uint32_t* tri;    // triangle of each record (wide == 0)
    const AccelRecWide* recw;  // 32-byte records (wide == 1)
    const AccelRecFull* recf;  // 64-byte records (wide == 2)
    uint32_t nf;            // fine cells per axis
    float invLf;            // nf / 2
    uint32_t wide;
};
// spin state reordered by cell; id = the spin's stable index
struct SpinsSorted {
    float *x, *y, *z, *mag, *phase;
    uint32_t *meta, *id;
    uint32_t N;
};
__host__ __device__ inline uint32_t accel_keys(uint32_t nf) {
    uint32_t v = nf - 1, s = 0;
    for (uint32_t b = 0; b < 10; b++) s |= ((v >> b) & 1u) << (3 * b);
    return (s | (s << 1) | (s << 2)) + 1;
}
int launch_accel_cells(bool fill, uint32_t nT, const TriPlane* plane, const TriBary* bary,
                       uint32_t nf, uint32_t* counter, const uint32_t* start, AccelRec* rec,
                       uint32_t* tri, AccelRecWide* recw, cudaStream_t st, AccelRecFull* recf = nullptr);
int launch_sort_spins(const SpinsSorted& S, const SpinsSorted& D, uint32_t nb, uint32_t* keys,
                      uint32_t* hist, uint32_t* start, uint32_t* scratch, cudaStream_t st);
int launch_unpermute(const SpinsSorted& S, const SpinsSorted& D, cudaStream_t st);
// flat.cu: the mesh step (warp-flattened candidate lists); occupancy 4, 6 or
// 8 blocks per SM; queue: plane-test survivors finished 32 at a time; stage:
// each cell's records staged in shared memory by bulk (TMA) copies
int launch_mesh_step_flat(const MeshDev& g, const AccelDev& acc, const MeshStepArgs& a,
                          const SpinsSorted& S, int rng, cudaStream_t st, int occupancy = 8,
                          bool queue = false, bool stage = false);
int launch_aos_to_soa(const float* pos, const void* spin, const SpinsSorted& D, cudaStream_t st);
int launch_soa_to_aos(const SpinsSorted& S, float* pos, void* spin, uint32_t* spinKeys,
                      uint32_t iterations, cudaStream_t st);

// ---- mesh.cu --------------------------------------------------------------
int launch_records_from_mesh(uint32_t nT, const float* V, const uint32_t* trgls,
                             const uint32_t* membrane, const uint32_t* fiber, TriPlane* plane,
                             TriBary* bary, cudaStream_t st);
int launch_tri64(uint32_t nT, const float* V, const uint32_t* trgls, Tri64* out, cudaStream_t st);
// every triangle's reference cells from the cell lists: up to 4 in a uint4
// (unused entries kCellNone), kCellMany in every entry when there are more
static constexpr uint32_t kCellNone = 0xFFFFFFFFu, kCellMany = 0xFFFFFFFEu;
int launch_tri_cell_lists(uint32_t ncells, uint32_t nT, const uint32_t* cell_start, const uint32_t* cell_tri,
                          uint32_t* count, uint4* out, cudaStream_t st);
int launch_records_from_helpers(uint32_t nT, const float* V, const float* H,
                                const uint32_t* triInfo, TriPlane* plane, TriBary* bary,
                                cudaStream_t st);
int launch_tri_cells(bool fill, uint32_t nT, const float* V, const uint32_t* trgls, uint32_t n,
                     float L, uint32_t* counter, const uint32_t* start, uint32_t* cell_tri,
                     cudaStream_t st);
int launch_sort_cells(uint32_t ncells, const uint32_t* start, uint32_t* cell_tri, cudaStream_t st);
int launch_dense_to_csr(uint32_t ncells, uint32_t maxTPC, uint32_t nT, const uint32_t* counter,
                        const uint32_t* dense, const uint32_t* start, uint32_t* cell_tri,
                        uint32_t* status, cudaStream_t st);

// ---- cyl.cu: the reference's cylinder grid on the GPU ----------------------
// counter[n^3] and cubes[n^3 * maxFPC] (addEntities order), cubeF (optional):
// each entry's fiber record; *maxCount: the fullest cell.  kErrGridOverflow
// when a cell needs more than maxFPC entries (the reference's build() fails).
int build_cyl_grid_gpu(const float4* fibers, uint32_t nF, uint32_t n, uint32_t maxFPC, float L, float maxR,
                       uint32_t* counter, uint32_t* cubes, float4* cubeF, uint32_t* maxCount, cudaStream_t st);

// ---- compartments.cu ------------------------------------------------------
int launch_compartments(const MeshDev& g, const AccelDev& acc, const SpinsSorted& S, const float maxabs[3],
                        float startBox, uint64_t seed, uint32_t maxTries, uint32_t maxMoves, uint32_t* status,
                        uint32_t* moved, cudaStream_t st);

// ---- scan.cu --------------------------------------------------------------
// content hashes of n device arrays of 32-bit words (nwords[k] words at
// ptrs[k]) into hostOut[n]; dOut is n device words of scratch.  Synchronous.
int hash_device_arrays(const void* const* ptrs, const size_t* nwords, int n, unsigned long long* dOut,
                       uint64_t* hostOut, cudaStream_t st);
// exclusive prefix sum: out[0..n] (out[n] = total); scratch >= scan_scratch_words(n)
size_t scan_scratch_words(uint32_t n);
int launch_scan_exclusive(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* scratch,
                          cudaStream_t st);

// ---- reduce.cu ------------------------------------------------------------
// Ensemble signal in FP64: out[c] = {sum m cos(phi), sum m sin(phi), count}
// for c = 0 (all spins) and 1 + compartment.  region > 0 keeps only spins
// with |x|,|y|,|z| < region (dSim2's getMrSignal).  partials: scratch of
// reduce_scratch_doubles(N) doubles.
size_t reduce_scratch_doubles(uint32_t N);
int launch_signal(const SpinsDev& S, int layout, double region, double* partials, double* out15,
                  cudaStream_t st);
// same partial pass over nb blocks (partials: nb * 15 doubles), then a
// warp-per-field final pass
int launch_signal_blocks(const SpinsDev& S, int layout, double region, double* partials, int nb,
                         double* out15, cudaStream_t st);

// ---- cyl.cu ---------------------------------------------------------------
struct CylDev {
    const float4* fibers;       // {x, y, z, r^2}; the axis coordinate is 2.0
    const uint32_t* cube_count; // dense reference grid (dSim2 addEntities)
    const uint32_t* cubes;
    const float4* cube_fibers;  // per grid entry, its fiber's record inline (or null)
    uint32_t n, maxFPC;
    float L;
    uint32_t nF;                // number of fibers (index bound)
    // fine filter grid (or null): each grid cell split fineK^3 ways; a fine
    // cell lists, in list order, the positions of its grid cell's entries
    // whose fiber can contain a point of the fine cell
    const uint32_t* fine_start; // (n fineK)^3 + 1 offsets
    const float4* fine_rec;     // per fine entry, the fiber record
    const uint32_t* fine_pos;   // per fine entry, its position in the grid cell's list
    uint32_t fineK;
    float fineInv;              // fineK / L
};
struct CylSpinsDev {
    float4* pos;       // x, y, z, phase (dSim2 GPU layout)
    uint32_t* seed4;   // s0, s1, imo + 1 (0 = derive from w), inside fiber / nearest
    float* mag;        // or null (no T2 in the dSim2 GPU ABI)
    uint32_t N;
};
struct CylStepArgs {
    float intraSd, extraSd, myelinSd;
    float T2fiber, T2myelin, T2outside;
    float perm, inRadPropSq;
    float clampHi, clampLo;
    float dt, pc;
    float gx, gy, gz;
    const float4* grad;
    uint32_t iterations;
    uint32_t key0, key1;
    uint64_t step0;
    uint32_t stream;
    const float4* draws;
    uint32_t* status;
    uint32_t* counts;
    uint32_t spinBase;    // added to the spin index in the Philox counter (replica shards)
};
// rng: kRngPhilox (key0/key1), kRngPhiloxPerSpinKey (seed4.x/.y), kRngReplay
int launch_cyl_step(const CylDev& g, const CylStepArgs& a, const CylSpinsDev& S, int rng,
                    cudaStream_t st);

// ---- host helpers --------------------------------------------------------
const char* last_error_message();
// api.cu: device views of native substrate handles (for batch.cu)
int mesh_views(const ::dsim_mesh* m, MeshDev* g, AccelDev* a);
// builds the mesh's FP64 triangle table on first use (kept until the mesh is freed)
int mesh_tri64(::dsim_mesh* m);
int cyl_view(const ::dsim_cyl* c, CylDev* g);
// fine filter grid of a reference cylinder grid (cyl.cu), built on the host
uint32_t cyl_fine_size(uint32_t n, float L, double maxR);
int cyl_fine_lists(const float* fiberPos, uint32_t nF, uint32_t n, uint32_t maxFPC, float cubeLength,
                   const uint32_t* cubeCounter, const uint32_t* cubes, uint32_t k, std::vector<uint32_t>& start,
                   std::vector<uint32_t>& pos, std::vector<float>& rec);
// batches holding a cylinder substrate's device view (+1 on add, -1 on free)
void cyl_hold(const ::dsim_cyl* c, int delta);
int mesh_rebuild_accel(::dsim_mesh* m, uint32_t nf);

}  // namespace dsim
