// batch.cu -- many simulation jobs advanced by one step launch per chunk
// (include/dsim_batch.h).
//
// Spins of all jobs live in one packed SoA array; job j owns the slot range
// [slot0_j, slot0_j + pad_j) with pad_j = nSpins rounded up to 32, so every
// warp belongs to one job and reads that job's substrate and parameters once.
// Padding slots carry id 0xFFFFFFFF and do no work.  Every chunk the spins
// are re-sorted by (job, Morton cell of a per-job sort grid) -- the job
// ranges are preserved because job j's keys follow job j-1's -- and one step
// kernel advances every running job by up to `chunk` steps.  The chunk loop
// (sort, step, step-counter advance) is captured in a CUDA graph.
//
// Step rules: mesh jobs run the flattened collision round of flat_round.cuh
// (dSim3/src/spinKernelCpu.cpp:198-499), cylinder jobs the dSim2 rules of
// cyl_common.cuh (dSim2/src/spinKernelCpu.cpp:312-641).  Draws are Philox with
// key = job seed and counter = (spin index in the job, job step, 0), the same
// as dsim_mesh_run / dsim_cyl_run with that seed.  Instead of the reference's
// float phase (dSim3/src/spinKernelCpu.cpp:490) each spin accumulates the
// gradient moment M = sum w(t) pos(t) with Kahan compensation; the phase of any
// gradient sharing the waveform is phaseConstant * (g . M), in FP64 at readout.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#pragma GCC visibility push(default)
#include "../../include/dsim_batch.h"
#pragma GCC visibility pop
#include "common.cuh"
#include "cyl_common.cuh"
#include "engine.h"
#include "flat_round.cuh"
#include "local_round.cuh"
#include "prec_round.cuh"

namespace dsim {

enum SubKind : uint32_t { kSubMesh = 0, kSubCyl = 1 };
struct SubDev {
    uint32_t kind;
    MeshDev g;
    AccelDev acc;
    CylDev c;
};

struct JobDev {
    uint32_t sub, steps, start;  // substrate, total steps, global step of the job's step 0
    uint32_t sortBase, sortBits;  // first sort key, Morton bits per axis of the sort grid
    float sd[4], T2[4];
    float perm, dt, clampHi, clampLo;
    uint32_t reflType, maxSub;
    float inR;                    // cylinders: (inner radius proportion)^2
    const float* wave;            // w[steps]
    uint32_t key0, key1;
    uint32_t flags;               // DSIM_JOB_PRECISE or DSIM_JOB_LOCAL
    float spinR;                  // spin radius (the precision form clamps to +-(1 - spinR) in FP64)
    uint32_t sortRegion;          // cylinders: spins outside every fiber sort after those inside
};

static_assert(sizeof(JobDev) % 4 == 0 && sizeof(SubDev) % 4 == 0, "records are copied by 32-bit words");

// packed spin state; meta = compartment | fiber << 8 (cylinders: imo | nearest << 8)
static constexpr int kBF = 10;  // float fields: x y z mx my mz cx cy cz mag
static constexpr int kBU = 3;   // uint fields: meta job id
static constexpr int kBD = 4;   // double fields of precision-form jobs: x y z mag (null until the first one)
struct BatchSpins {
    float* f[kBF];
    uint32_t* u[kBU];
    double* d[kBD];
    uint32_t N;
};
enum { F_X, F_Y, F_Z, F_MX, F_MY, F_MZ, F_CX, F_CY, F_CZ, F_MAG };
enum { U_META, U_JOB, U_ID };
enum { D_X, D_Y, D_Z, D_MAG };

__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}

// The plain form has one instantiation per fine-grid record layout (LAYOUT 1:
// 32-byte, 2: 64-byte records), each advancing only the mesh jobs whose
// substrate uses it, and one for cylinder jobs (LAYOUT 3), so no kernel
// carries the registers of a path it does not run.  Precision-form and
// cell-local jobs run in k_batch_step64 and k_batch_step_local.  THREADS:
// block size (64, 128 or 256); MINB counts 128-thread blocks per SM, so every
// block shape of one occupancy has the same register budget per thread.
template <int MINB, int LAYOUT, int THREADS = kFlatThreads>
__global__ void __launch_bounds__(THREADS, MINB * kFlatThreads / THREADS)
k_batch_step(const SubDev* __restrict__ subs, const JobDev* __restrict__ jobs, BatchSpins S,
             const uint32_t* __restrict__ stepNow, uint32_t chunk, uint32_t* status,
             unsigned long long* jobCounts) {
    constexpr int MESH = LAYOUT == 3 ? 1 : LAYOUT;  // the record path of the mesh instantiations
    __shared__ FlatWarp wh[LAYOUT == 3 ? 1 : THREADS / 32];
    // gradient moments and their compensation live in shared memory (touched
    // once per step), which keeps the collision loop's registers free
    __shared__ float mom[6][THREADS];
    const uint32_t FULL = 0xFFFFFFFFu;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t tx = threadIdx.x;
    FlatWarp& H = wh[LAYOUT == 3 ? 0u : (threadIdx.x >> 5)];  // the cylinder path uses no table
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if ((i & ~31u) >= S.N) return;  // whole warp: N is a multiple of 32
    const uint32_t jb = S.u[U_JOB][i & ~31u];
    // the warp's job and substrate records, copied to shared memory once and
    // read from there (kept out of the collision loop's registers)
    __shared__ JobDev jobS[THREADS / 32];
    __shared__ SubDev subS[THREADS / 32];
    const uint32_t wi = threadIdx.x >> 5;
    {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(jobs + jb);
        uint32_t* dst = reinterpret_cast<uint32_t*>(jobS + wi);
        for (uint32_t k = lane; k < sizeof(JobDev) / 4; k += 32) dst[k] = __ldg(src + k);
        __syncwarp();
        const uint32_t* s2 = reinterpret_cast<const uint32_t*>(subs + jobS[wi].sub);
        uint32_t* d2 = reinterpret_cast<uint32_t*>(subS + wi);
        for (uint32_t k = lane; k < sizeof(SubDev) / 4; k += 32) d2[k] = __ldg(s2 + k);
        __syncwarp();
    }
    const JobDev& J = jobS[wi];
    if (J.flags & (DSIM_JOB_PRECISE | DSIM_JOB_LOCAL)) return;  // warp-uniform
    if (LAYOUT == 3 ? subS[wi].kind != kSubCyl
                    : (subS[wi].kind != kSubMesh || subS[wi].acc.wide != (uint32_t)LAYOUT)) return;
    const uint32_t now = *stepNow;
    const uint32_t start = J.start, steps = J.steps;
    if (now < start || now - start >= steps) return;  // not started or finished (warp-uniform)
    const uint32_t ls0 = now - start;
    const uint32_t nsteps = min(chunk, steps - ls0);
    const uint32_t id = S.u[U_ID][i];
    const bool valid = id != 0xFFFFFFFFu;
    float x = S.f[F_X][i], y = S.f[F_Y][i], z = S.f[F_Z][i];
    mom[0][tx] = S.f[F_MX][i]; mom[1][tx] = S.f[F_MY][i]; mom[2][tx] = S.f[F_MZ][i];
    mom[3][tx] = S.f[F_CX][i]; mom[4][tx] = S.f[F_CY][i]; mom[5][tx] = S.f[F_CZ][i];
    float mag = S.f[F_MAG][i];
    const uint32_t meta = S.u[U_META][i];
    uint32_t comp = meta & 0xFFu, fiber = meta >> 8;
    const uint32_t k0 = J.key0, k1 = J.key1;
    const float* __restrict__ wave = J.wave;
    uint32_t nrefl = 0, nperm = 0, st = 0;
    const SubDev& sub = subS[wi];
    if (LAYOUT != 3) {
        const MeshDev& g = sub.g;
        const AccelDev& acc = sub.acc;
        const float perm = J.perm;
        const uint32_t reflType = J.reflType, maxSub = J.maxSub;
        uint32_t it = 0;
        bool active = valid && nsteps > 0;
        bool fresh = active;
        Draw d;
        d.nx = d.ny = d.nz = 0.0f; d.u = 1.0f;
        float ox = x, oy = y, oz = z, px = x, py = y, pz = z;
        uint32_t excluded = 0xFFFFFFFFu, sub_n = 0;
        float umax = 1.0f, umin = 0.0f;
        while (__any_sync(FULL, active)) {
            if (fresh) {
                d = philox_draw(id, (uint64_t)(ls0 + it), 0u, k0, k1);
                ox = x; oy = y; oz = z;
                const float sd = J.sd[comp & 3u];
                px = x + d.nx * sd; py = y + d.ny * sd; pz = z + d.nz * sd;
                excluded = 0xFFFFFFFFu;
                umax = 1.0f; umin = 0.0f;
                sub_n = 0;
                fresh = false;
            }
            const bool open = active;
            bool found;
            FastHit best;
            flat_round_mode<MESH>(H, g, acc, lane, open, ox, oy, oz, px, py, pz, excluded, found, best);
            if (open) {
                bool finish = !found;
                if (found) {
                    apply_hit(g, best, d.u, perm, reflType, umax, umin, ox, oy, oz, px, py, pz, comp, fiber,
                              excluded, nrefl, nperm);
                    if (++sub_n >= maxSub) {
                        st |= kStatusSubsegCap;
                        px = ox; py = oy; pz = oz;
                        finish = true;
                    }
                }
                if (finish) {
                    float ex = px, ey = py, ez = pz;
                    if (ex > J.clampHi) ex = J.clampHi; else if (ex < J.clampLo) ex = J.clampLo;
                    if (ey > J.clampHi) ey = J.clampHi; else if (ey < J.clampLo) ey = J.clampLo;
                    if (ez > J.clampHi) ez = J.clampHi; else if (ez < J.clampLo) ez = J.clampLo;
                    x = ex; y = ey; z = ez;
                    const float T2 = J.T2[comp & 3u];
                    if (T2 > 0.0f) mag += -mag / T2 * J.dt;
                    const float w = __ldg(wave + ls0 + it);
                    kahan_add(mom[0][tx], mom[3][tx], w * x);
                    kahan_add(mom[1][tx], mom[4][tx], w * y);
                    kahan_add(mom[2][tx], mom[5][tx], w * z);
                    if (++it >= nsteps) active = false;
                    else fresh = true;
                }
            }
            __syncwarp();
        }
    } else if (valid) {
        const CylDev& g = sub.c;
        const float perm = J.perm, inR = J.inR;
        uint32_t imo = comp, nearest = fiber;
        if (imo < 2 && nearest >= g.nF) imo = 2;
        for (uint32_t it = 0; it < nsteps; it++) {
            const Draw d = philox_draw(id, (uint64_t)(ls0 + it), 0u, k0, k1);
            const float ox = x, oy = y, oz = z;
            const float sdv = J.sd[imo];
            float px = x + d.nx * sdv, py = y + d.ny * sdv, pz = z + d.nz * sdv;
            if (perm < 1.0f) cyl_membranes(g, ox, oy, oz, px, py, pz, d.u, perm, inR, imo, nearest, nrefl, nperm, st);
            if (px > J.clampHi) px = J.clampHi; else if (px < J.clampLo) px = J.clampLo;
            if (py > J.clampHi) py = J.clampHi; else if (py < J.clampLo) py = J.clampLo;
            if (pz > J.clampHi) pz = J.clampHi; else if (pz < J.clampLo) pz = J.clampLo;
            x = px; y = py; z = pz;
            const float T2 = J.T2[imo];
            if (T2 > 0.0f) mag += -mag / T2 * J.dt;
            const float w = __ldg(wave + ls0 + it);
            kahan_add(mom[0][tx], mom[3][tx], w * x);
            kahan_add(mom[1][tx], mom[4][tx], w * y);
            kahan_add(mom[2][tx], mom[5][tx], w * z);
        }
        comp = imo;
        fiber = nearest & 0xFFFFFFu;
    }
    if (valid) {
        S.f[F_X][i] = x; S.f[F_Y][i] = y; S.f[F_Z][i] = z;
        S.f[F_MX][i] = mom[0][tx]; S.f[F_MY][i] = mom[1][tx]; S.f[F_MZ][i] = mom[2][tx];
        S.f[F_CX][i] = mom[3][tx]; S.f[F_CY][i] = mom[4][tx]; S.f[F_CZ][i] = mom[5][tx];
        S.f[F_MAG][i] = mag;
        S.u[U_META][i] = (comp & 0xFFu) | (fiber << 8);
    }
    // per-job counters {reflections, permeations}: one atomic per warp
    unsigned long long r = nrefl, p = nperm;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        r += __shfl_down_sync(FULL, r, o);
        p += __shfl_down_sync(FULL, p, o);
    }
    if (lane == 0) {
        if (r) atomicAdd(jobCounts + 4 * jb, r);
        if (p) atomicAdd(jobCounts + 4 * jb + 1, p);
    }
    if (st) atomicOr(status, st);
}

// Cell-local FP32 mesh jobs (DSIM_JOB_LOCAL): the plain step with positions
// as FP32 offsets from a lattice origin (local_round.cuh), FP64 re-tests of
// near-degenerate intersections, Kahan moments.  Between chunks the position
// is kept in the double fields as origin + offset; the float fields get its
// rounded value (sort keys, float readers).
template <int LAYOUT>
__global__ void __launch_bounds__(kFlatThreads, 4)
k_batch_step_local(const SubDev* __restrict__ subs, const JobDev* __restrict__ jobs, BatchSpins S,
                   const uint32_t* __restrict__ stepNow, uint32_t chunk, uint32_t* status,
                   unsigned long long* jobCounts) {
    __shared__ FlatWarp wh[kFlatWarps];
    __shared__ LocalWarp wl[kFlatWarps];
    __shared__ float mom[6][kFlatThreads];
    __shared__ JobDev jobS[kFlatWarps];
    __shared__ SubDev subS[kFlatWarps];
    const uint32_t FULL = 0xFFFFFFFFu;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t tx = threadIdx.x;
    const uint32_t wi = threadIdx.x >> 5;
    FlatWarp& H = wh[wi];
    LocalWarp& Lw = wl[wi];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if ((i & ~31u) >= S.N) return;  // whole warp: N is a multiple of 32
    const uint32_t jb = S.u[U_JOB][i & ~31u];
    {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(jobs + jb);
        uint32_t* dst = reinterpret_cast<uint32_t*>(jobS + wi);
        for (uint32_t k = lane; k < sizeof(JobDev) / 4; k += 32) dst[k] = __ldg(src + k);
        __syncwarp();
        const uint32_t* s2 = reinterpret_cast<const uint32_t*>(subs + jobS[wi].sub);
        uint32_t* d2 = reinterpret_cast<uint32_t*>(subS + wi);
        for (uint32_t k = lane; k < sizeof(SubDev) / 4; k += 32) d2[k] = __ldg(s2 + k);
        __syncwarp();
    }
    const JobDev& J = jobS[wi];
    if (!(J.flags & DSIM_JOB_LOCAL) || subS[wi].kind != kSubMesh || subS[wi].acc.wide != (uint32_t)LAYOUT)
        return;  // warp-uniform
    const uint32_t now = *stepNow;
    const uint32_t start = J.start, steps = J.steps;
    if (now < start || now - start >= steps) return;
    const uint32_t ls0 = now - start;
    const uint32_t nsteps = min(chunk, steps - ls0);
    const uint32_t id = S.u[U_ID][i];
    const bool valid = id != 0xFFFFFFFFu;
    // position = lattice origin (multiple of 1/16) + FP32 offset in [0, 1/16)
    float gx = 0.0f, gy = 0.0f, gz = 0.0f, x = 0.0f, y = 0.0f, z = 0.0f, mag = 0.0f;
    uint32_t comp = 0, fiber = 0;
    mom[0][tx] = 0.0f; mom[1][tx] = 0.0f; mom[2][tx] = 0.0f;
    mom[3][tx] = 0.0f; mom[4][tx] = 0.0f; mom[5][tx] = 0.0f;
    if (valid) {
        const double X = S.d[D_X][i], Y = S.d[D_Y][i], Z = S.d[D_Z][i];
        const double Gx = floor(X * 16.0) * 0.0625, Gy = floor(Y * 16.0) * 0.0625, Gz = floor(Z * 16.0) * 0.0625;
        gx = (float)Gx; gy = (float)Gy; gz = (float)Gz;
        x = (float)(X - Gx); y = (float)(Y - Gy); z = (float)(Z - Gz);
        mag = S.f[F_MAG][i];
        mom[0][tx] = S.f[F_MX][i]; mom[1][tx] = S.f[F_MY][i]; mom[2][tx] = S.f[F_MZ][i];
        mom[3][tx] = S.f[F_CX][i]; mom[4][tx] = S.f[F_CY][i]; mom[5][tx] = S.f[F_CZ][i];
        const uint32_t meta = S.u[U_META][i];
        comp = meta & 0xFFu; fiber = meta >> 8;
    }
    const MeshDev& g = subS[wi].g;
    const AccelDev& acc = subS[wi].acc;
    const float perm = J.perm;
    const uint32_t reflType = J.reflType, maxSub = J.maxSub;
    const uint32_t k0 = J.key0, k1 = J.key1;
    const float* __restrict__ wave = J.wave;
    uint32_t nrefl = 0, nperm = 0, st = 0, it = 0, excluded = 0xFFFFFFFFu, sub_n = 0;
    PrecCount pc;
    bool active = valid && nsteps > 0;
    bool fresh = active;
    Draw d;
    d.nx = d.ny = d.nz = 0.0f; d.u = 1.0f;
    float umax = 1.0f, umin = 0.0f;
    float ox = x, oy = y, oz = z, px = x, py = y, pz = z;
    while (__any_sync(FULL, active)) {
        if (fresh) {
            d = philox_draw(id, (uint64_t)(ls0 + it), 0u, k0, k1);
            ox = x; oy = y; oz = z;
            const float sd = J.sd[comp & 3u];
            px = x + d.nx * sd; py = y + d.ny * sd; pz = z + d.nz * sd;
            excluded = 0xFFFFFFFFu;
            umax = 1.0f; umin = 0.0f;
            sub_n = 0;
            fresh = false;
        }
        const bool open = active;
        bool found;
        FastHit best;
        local_round<LAYOUT>(H, Lw, g, acc, lane, open, gx, gy, gz, ox, oy, oz, px, py, pz, excluded, found, best, pc);
        if (open) {
            bool finish = !found;
            if (found) {
                apply_hit(g, best, d.u, perm, reflType, umax, umin, ox, oy, oz, px, py, pz, comp, fiber, excluded,
                          nrefl, nperm);
                if (++sub_n >= maxSub) {
                    st |= kStatusSubsegCap;
                    px = ox; py = oy; pz = oz;
                    finish = true;
                }
            }
            if (finish) {
                // clamp in absolute coordinates, then move the origin so the
                // offset is back in [0, 1/16)
                float ax = gx + px, ay = gy + py, az = gz + pz;
                if (ax > J.clampHi) px = J.clampHi - gx; else if (ax < J.clampLo) px = J.clampLo - gx;
                if (ay > J.clampHi) py = J.clampHi - gy; else if (ay < J.clampLo) py = J.clampLo - gy;
                if (az > J.clampHi) pz = J.clampHi - gz; else if (az < J.clampLo) pz = J.clampLo - gz;
                const float sx = floor_small(px * 16.0f) * kLatticeH, sy = floor_small(py * 16.0f) * kLatticeH,
                            sz = floor_small(pz * 16.0f) * kLatticeH;
                gx += sx; gy += sy; gz += sz;
                x = px - sx; y = py - sy; z = pz - sz;
                const float T2 = J.T2[comp & 3u];
                if (T2 > 0.0f) mag += -mag / T2 * J.dt;
                const float w = __ldg(wave + ls0 + it);
                kahan_add(mom[0][tx], mom[3][tx], w * (gx + x));
                kahan_add(mom[1][tx], mom[4][tx], w * (gy + y));
                kahan_add(mom[2][tx], mom[5][tx], w * (gz + z));
                if (++it >= nsteps) active = false;
                else fresh = true;
            }
        }
        __syncwarp();
    }
    if (valid) {
        const double X = (double)gx + (double)x, Y = (double)gy + (double)y, Z = (double)gz + (double)z;
        S.d[D_X][i] = X; S.d[D_Y][i] = Y; S.d[D_Z][i] = Z; S.d[D_MAG][i] = (double)mag;
        S.f[F_X][i] = (float)X; S.f[F_Y][i] = (float)Y; S.f[F_Z][i] = (float)Z;
        S.f[F_MAG][i] = mag;
        S.f[F_MX][i] = mom[0][tx]; S.f[F_MY][i] = mom[1][tx]; S.f[F_MZ][i] = mom[2][tx];
        S.f[F_CX][i] = mom[3][tx]; S.f[F_CY][i] = mom[4][tx]; S.f[F_CZ][i] = mom[5][tx];
        S.u[U_META][i] = (comp & 0xFFu) | (fiber << 8);
    }
    // per-job counters {reflections, permeations, records examined, FP64 re-tests}
    unsigned long long r = nrefl, p = nperm, te = pc.records, ex = pc.exact;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        r += __shfl_down_sync(FULL, r, o);
        p += __shfl_down_sync(FULL, p, o);
        te += __shfl_down_sync(FULL, te, o);
        ex += __shfl_down_sync(FULL, ex, o);
    }
    if (lane == 0) {
        if (r) atomicAdd(jobCounts + 4 * jb, r);
        if (p) atomicAdd(jobCounts + 4 * jb + 1, p);
        if (te) atomicAdd(jobCounts + 4 * jb + 2, te);
        if (ex) atomicAdd(jobCounts + 4 * jb + 3, ex);
    }
    if (st) atomicOr(status, st);
}

// Precision-form mesh jobs (DSIM_JOB_PRECISE): the step of cpuIntegrate
// (dSim3/src/spinKernelCpu.cpp:430-499) in FP64 -- position, sub-segments,
// hits and reflections (prec_round.cuh), the clamp to +-(1 - spinRadius), the
// T2 decay and the gradient moments M += w(t) pos(t) -- on the same Philox
// draws as the plain form.  Positions and magnitudes persist in the double
// fields; the float fields receive their rounded values (sort keys, float
// readers) and the moment pair (m, c) holds M as m - c.
__global__ void __launch_bounds__(kFlatThreads, 2)
k_batch_step64(const SubDev* __restrict__ subs, const JobDev* __restrict__ jobs, BatchSpins S,
               const uint32_t* __restrict__ stepNow, uint32_t chunk, uint32_t* status,
               unsigned long long* jobCounts) {
    __shared__ FlatWarp wh[kFlatWarps];
    __shared__ PrecWarp wp[kFlatWarps];
    __shared__ JobDev jobS[kFlatWarps];
    __shared__ SubDev subS[kFlatWarps];
    const uint32_t FULL = 0xFFFFFFFFu;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t wi = threadIdx.x >> 5;
    FlatWarp& H = wh[wi];
    PrecWarp& P = wp[wi];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if ((i & ~31u) >= S.N) return;  // whole warp: N is a multiple of 32
    const uint32_t jb = S.u[U_JOB][i & ~31u];
    {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(jobs + jb);
        uint32_t* dst = reinterpret_cast<uint32_t*>(jobS + wi);
        for (uint32_t k = lane; k < sizeof(JobDev) / 4; k += 32) dst[k] = __ldg(src + k);
        __syncwarp();
        const uint32_t* s2 = reinterpret_cast<const uint32_t*>(subs + jobS[wi].sub);
        uint32_t* d2 = reinterpret_cast<uint32_t*>(subS + wi);
        for (uint32_t k = lane; k < sizeof(SubDev) / 4; k += 32) d2[k] = __ldg(s2 + k);
        __syncwarp();
    }
    const JobDev& J = jobS[wi];
    if (!(J.flags & DSIM_JOB_PRECISE) || subS[wi].kind != kSubMesh) return;  // warp-uniform
    const uint32_t now = *stepNow;
    const uint32_t start = J.start, steps = J.steps;
    if (now < start || now - start >= steps) return;
    const uint32_t ls0 = now - start;
    const uint32_t nsteps = min(chunk, steps - ls0);
    const uint32_t id = S.u[U_ID][i];
    const bool valid = id != 0xFFFFFFFFu;
    double x = 0.0, y = 0.0, z = 0.0, mag = 0.0, Mx = 0.0, My = 0.0, Mz = 0.0;
    uint32_t comp = 0, fiber = 0;
    if (valid) {
        x = S.d[D_X][i]; y = S.d[D_Y][i]; z = S.d[D_Z][i]; mag = S.d[D_MAG][i];
        Mx = (double)S.f[F_MX][i] - (double)S.f[F_CX][i];
        My = (double)S.f[F_MY][i] - (double)S.f[F_CY][i];
        Mz = (double)S.f[F_MZ][i] - (double)S.f[F_CZ][i];
        const uint32_t meta = S.u[U_META][i];
        comp = meta & 0xFFu; fiber = meta >> 8;
    }
    const MeshDev& g = subS[wi].g;
    const AccelDev& acc = subS[wi].acc;
    const double perm = (double)J.perm;
    const double hiC = 1.0 - (double)J.spinR, loC = -1.0 + (double)J.spinR;
    const uint32_t reflType = J.reflType, maxSub = J.maxSub;
    const uint32_t k0 = J.key0, k1 = J.key1;
    const float* __restrict__ wave = J.wave;
    uint32_t nrefl = 0, nperm = 0, st = 0, it = 0, excluded = 0xFFFFFFFFu, sub_n = 0;
    PrecCount pc;
    bool active = valid && nsteps > 0;
    bool fresh = active;
    double u = 1.0, umax = 1.0, umin = 0.0;
    double ox = x, oy = y, oz = z, px = x, py = y, pz = z;
    while (__any_sync(FULL, active)) {
        if (fresh) {
            const Draw d = philox_draw(id, (uint64_t)(ls0 + it), 0u, k0, k1);
            ox = x; oy = y; oz = z;
            const double sd = (double)J.sd[comp & 3u];
            px = x + (double)d.nx * sd; py = y + (double)d.ny * sd; pz = z + (double)d.nz * sd;
            u = (double)d.u;
            excluded = 0xFFFFFFFFu;
            umax = 1.0; umin = 0.0;
            sub_n = 0;
            fresh = false;
        }
        const bool open = active;
        bool found;
        uint32_t ht = 0, htype = 0;
        double hx = 0.0, hy = 0.0, hz = 0.0;
        prec_round(H, P, g, acc, lane, open, ox, oy, oz, px, py, pz, excluded, found, ht, htype, hx, hy, hz, pc);
        if (open) {
            bool finish = !found;
            if (found) {
                apply_hit64(g, ht, htype, hx, hy, hz, u, perm, reflType, umax, umin, ox, oy, oz, px, py, pz, comp,
                            fiber, excluded, nrefl, nperm);
                if (++sub_n >= maxSub) {
                    st |= kStatusSubsegCap;
                    px = ox; py = oy; pz = oz;
                    finish = true;
                }
            }
            if (finish) {
                if (px > hiC) px = hiC; else if (px < loC) px = loC;
                if (py > hiC) py = hiC; else if (py < loC) py = loC;
                if (pz > hiC) pz = hiC; else if (pz < loC) pz = loC;
                x = px; y = py; z = pz;
                const float T2 = J.T2[comp & 3u];
                if (T2 > 0.0f) mag += -mag / (double)T2 * (double)J.dt;
                const double w = (double)__ldg(wave + ls0 + it);
                Mx += w * x; My += w * y; Mz += w * z;
                if (++it >= nsteps) active = false;
                else fresh = true;
            }
        }
        __syncwarp();
    }
    if (valid) {
        S.d[D_X][i] = x; S.d[D_Y][i] = y; S.d[D_Z][i] = z; S.d[D_MAG][i] = mag;
        S.f[F_X][i] = (float)x; S.f[F_Y][i] = (float)y; S.f[F_Z][i] = (float)z;
        S.f[F_MAG][i] = (float)mag;
        const float mx = (float)Mx, my = (float)My, mz = (float)Mz;
        S.f[F_MX][i] = mx; S.f[F_MY][i] = my; S.f[F_MZ][i] = mz;
        S.f[F_CX][i] = (float)((double)mx - Mx);
        S.f[F_CY][i] = (float)((double)my - My);
        S.f[F_CZ][i] = (float)((double)mz - Mz);
        S.u[U_META][i] = (comp & 0xFFu) | (fiber << 8);
    }
    // per-job counters {reflections, permeations, records examined, FP64 triangle tests}
    unsigned long long r = nrefl, p = nperm, te = pc.records, ex = pc.exact;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        r += __shfl_down_sync(FULL, r, o);
        p += __shfl_down_sync(FULL, p, o);
        te += __shfl_down_sync(FULL, te, o);
        ex += __shfl_down_sync(FULL, ex, o);
    }
    if (lane == 0) {
        if (r) atomicAdd(jobCounts + 4 * jb, r);
        if (p) atomicAdd(jobCounts + 4 * jb + 1, p);
        if (te) atomicAdd(jobCounts + 4 * jb + 2, te);
        if (ex) atomicAdd(jobCounts + 4 * jb + 3, ex);
    }
    if (st) atomicOr(status, st);
}

__global__ void k_batch_advance(uint32_t* stepNow, uint32_t chunk) { *stepNow += chunk; }

// sort key: job's base + Morton code of the spin's cell in a 2^bits grid
// over the box; padding goes to the job's last key
__global__ void k_batch_keys(const JobDev* __restrict__ jobs, BatchSpins S, uint32_t* keys,
                             uint32_t* hist) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.N) return;
    const JobDev& J = jobs[S.u[U_JOB][i]];
    const uint32_t bits = J.sortBits, n = 1u << bits;
    uint32_t key;
    if (S.u[U_ID][i] == 0xFFFFFFFFu) {
        key = J.sortBase + ((J.sortRegion ? 2u : 1u) << (3 * bits)) - 1u;
    } else {
        // cylinder jobs: a spin outside every fiber scans its cell's fiber
        // list (twice), one inside tests its own fiber once, so the two
        // kinds go to separate warps: region (imo == 2) above the cell code
        const uint32_t region = J.sortRegion && (S.u[U_META][i] & 0xFFu) >= 2u ? 1u : 0u;
        const float s = 0.5f * (float)n;
        uint32_t a = (uint32_t)fminf(fmaxf(floorf((S.f[F_X][i] + 1.0f) * s), 0.0f), (float)(n - 1));
        uint32_t b = (uint32_t)fminf(fmaxf(floorf((S.f[F_Y][i] + 1.0f) * s), 0.0f), (float)(n - 1));
        uint32_t c = (uint32_t)fminf(fmaxf(floorf((S.f[F_Z][i] + 1.0f) * s), 0.0f), (float)(n - 1));
        key = J.sortBase + (region << (3 * bits)) + morton3(a, b, c);
    }
    keys[i] = key;
    atomicAdd(hist + key, 1u);
}

__global__ void k_batch_scatter(BatchSpins S, BatchSpins D, const uint32_t* __restrict__ keys,
                                const uint32_t* __restrict__ start, uint32_t* cursor) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.N) return;
    const uint32_t k = keys[i];
    const uint32_t j = start[k] + atomicAdd(cursor + k, 1u);
#pragma unroll
    for (int f = 0; f < kBF; f++) D.f[f][j] = S.f[f][i];
#pragma unroll
    for (int u = 0; u < kBU; u++) D.u[u][j] = S.u[u][i];
    if (S.d[0]) {
#pragma unroll
        for (int f = 0; f < kBD; f++) D.d[f][j] = S.d[f][i];
    }
}

// compaction: slot i of a kept job moves to remapped slot; job index remapped
__global__ void k_batch_compact(BatchSpins S, BatchSpins D, const int32_t* __restrict__ jobMap,
                                const int64_t* __restrict__ slotShift) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.N) return;
    const uint32_t jb = S.u[U_JOB][i];
    const int32_t nj = jobMap[jb];
    if (nj < 0) return;
    const uint32_t j = (uint32_t)((int64_t)i + slotShift[jb]);
#pragma unroll
    for (int f = 0; f < kBF; f++) D.f[f][j] = S.f[f][i];
    D.u[U_META][j] = S.u[U_META][i];
    D.u[U_JOB][j] = (uint32_t)nj;
    D.u[U_ID][j] = S.u[U_ID][i];
    if (S.d[0]) {
#pragma unroll
        for (int f = 0; f < kBD; f++) D.d[f][j] = S.d[f][i];
    }
}

// a job's spins in spin order
__global__ void k_batch_gather(BatchSpins S, uint32_t slot0, uint32_t len, float* pos3, float* mag,
                               float* mom6, uint32_t* meta) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= len) return;
    const uint32_t i = slot0 + k;
    const uint32_t id = S.u[U_ID][i];
    if (id == 0xFFFFFFFFu) return;
    pos3[3 * id] = S.f[F_X][i]; pos3[3 * id + 1] = S.f[F_Y][i]; pos3[3 * id + 2] = S.f[F_Z][i];
    mag[id] = S.f[F_MAG][i];
    mom6[6 * id] = S.f[F_MX][i]; mom6[6 * id + 1] = S.f[F_MY][i]; mom6[6 * id + 2] = S.f[F_MZ][i];
    mom6[6 * id + 3] = S.f[F_CX][i]; mom6[6 * id + 4] = S.f[F_CY][i]; mom6[6 * id + 5] = S.f[F_CZ][i];
    meta[id] = S.u[U_META][i];
}

// a precision-form job's FP64 positions and magnitudes in spin order
__global__ void k_batch_gather64(BatchSpins S, uint32_t slot0, uint32_t len, double* pos3, double* mag) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= len) return;
    const uint32_t i = slot0 + k;
    const uint32_t id = S.u[U_ID][i];
    if (id == 0xFFFFFFFFu) return;
    pos3[3 * id] = S.d[D_X][i]; pos3[3 * id + 1] = S.d[D_Y][i]; pos3[3 * id + 2] = S.d[D_Z][i];
    mag[id] = S.d[D_MAG][i];
}

// FP64 signal of one job for nG gradients: partial records per (block, g)
static constexpr int kSigThreads = 128;
// Readout of one job for nG gradients sharing its waveform.  Warp w takes
// the 32 gradients [32 (w % gw), 32 (w % gw) + 32) and the spins of segment
// w / gw (contiguous slots): its lanes read each spin once (one address: a
// broadcast load) and each lane keeps its own gradient's sums in registers,
// so no per-gradient reduction across threads is needed.  partials[segment]
// [gradient][15] = {X, Y, n} for all spins and per compartment, each summed in
// slot order; k_batch_signal_final adds the segments in order, so the result
// does not depend on the launch.  fp64: the job keeps FP64 positions and
// magnitudes (precision and cell-local forms), which the readout then uses.
__global__ void __launch_bounds__(kSigThreads) k_batch_signal(BatchSpins S, uint32_t slot0, uint32_t len,
                                                              const double* __restrict__ kg, uint32_t nG,
                                                              uint32_t gw, uint32_t nseg, uint32_t segLen,
                                                              double region, bool fp64, double* partials) {
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (warp >= gw * nseg) return;  // whole warps
    const uint32_t gi = (warp % gw) * 32u + lane, sg = warp / gw;
    const bool live = gi < nG;
    const double gx = live ? kg[3 * gi] : 0.0, gy = live ? kg[3 * gi + 1] : 0.0, gz = live ? kg[3 * gi + 2] : 0.0;
    double X = 0.0, Y = 0.0, cX[4] = {0.0, 0.0, 0.0, 0.0}, cY[4] = {0.0, 0.0, 0.0, 0.0};
    uint32_t n = 0, cn[4] = {0u, 0u, 0u, 0u};
    const uint32_t k0 = sg * segLen, k1 = min(len, k0 + segLen);
    for (uint32_t k = k0; k < k1; k++) {  // the same spin on every lane: warp-uniform branches
        const uint32_t i = slot0 + k;
        if (S.u[U_ID][i] == 0xFFFFFFFFu) continue;
        if (region > 0.0) {  // dSim2's readout box (dSim2/src/spinSystem.cpp:944-978)
            const double x = fp64 ? S.d[D_X][i] : (double)S.f[F_X][i];
            const double y = fp64 ? S.d[D_Y][i] : (double)S.f[F_Y][i];
            const double z = fp64 ? S.d[D_Z][i] : (double)S.f[F_Z][i];
            if (!(x > -region && x < region && y > -region && y < region && z > -region && z < region)) continue;
        }
        const double Mx = (double)S.f[F_MX][i] - (double)S.f[F_CX][i];
        const double My = (double)S.f[F_MY][i] - (double)S.f[F_CY][i];
        const double Mz = (double)S.f[F_MZ][i] - (double)S.f[F_CZ][i];
        const double m = fp64 ? S.d[D_MAG][i] : (double)S.f[F_MAG][i];
        const uint32_t comp = S.u[U_META][i] & 3u;
        double sn, cs;
        sincos(gx * Mx + gy * My + gz * Mz, &sn, &cs);
        const double xs = m * cs, ys = m * sn;
        X += xs; Y += ys; n++;
        if (comp == 0) { cX[0] += xs; cY[0] += ys; cn[0]++; }
        else if (comp == 1) { cX[1] += xs; cY[1] += ys; cn[1]++; }
        else if (comp == 2) { cX[2] += xs; cY[2] += ys; cn[2]++; }
        else { cX[3] += xs; cY[3] += ys; cn[3]++; }
    }
    if (!live) return;
    double* o = partials + ((size_t)sg * nG + gi) * 15;
    o[0] = X; o[1] = Y; o[2] = (double)n;
#pragma unroll
    for (int q = 0; q < 4; q++) { o[3 + 3 * q] = cX[q]; o[4 + 3 * q] = cY[q]; o[5 + 3 * q] = (double)cn[q]; }
}

__global__ void k_batch_signal_final(const double* __restrict__ partials, uint32_t nb, uint32_t nG,
                                     double* out) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nG * 15) return;
    double v = 0.0;
    for (uint32_t b = 0; b < nb; b++) v += partials[(size_t)b * nG * 15 + t];
    out[t] = v;
}

}  // namespace dsim

using namespace dsim;

struct BatchBuf {
    float* f[kBF] = {};
    uint32_t* u[kBU] = {};
    double* d[kBD] = {};
};

struct BatchJob {
    uint32_t id;            // public job id
    JobDev d;
    uint32_t nSpins, pad;
    uint64_t slot0;
    float* wave = nullptr;  // device table
    double pc = 0.0;        // phase constant 2 pi gamma dt
    bool retired = false;
    uint64_t counts[2] = {0, 0};
};

struct dsim_batch {
    cudaStream_t st = nullptr;
    // the step kernels of a chunk (one per record layout and form) advance
    // disjoint jobs: they run side by side on these streams, forked from st
    // after the sort and joined before the step counter advances
    static constexpr int kSide = 6;
    cudaStream_t side[kSide] = {};
    cudaEvent_t forkEv = nullptr, joinEv[kSide] = {};
    uint64_t cap = 0;
    uint32_t jobCap = 0;
    BatchBuf buf[2];
    int cur = 0;
    uint64_t N = 0;
    std::vector<SubDev> subs;
    std::vector<const dsim_mesh*> meshes;  // per substrate (null for cylinders)
    std::vector<const dsim_cyl*> cylsHeld; // cylinder substrates added (released on free)
    SubDev* d_subs = nullptr;
    uint32_t subCap = 256;
    std::vector<BatchJob> jobs;            // packing order
    uint32_t nextId = 0;
    JobDev* d_jobs = nullptr;
    unsigned long long* d_counts = nullptr;
    uint32_t* d_status = nullptr;
    uint32_t* d_stepNow = nullptr;
    uint32_t stepNow = 0;                  // host mirror of *d_stepNow
    uint32_t* keys = nullptr;
    uint32_t *hist = nullptr, *hstart = nullptr, *scratch = nullptr;
    uint64_t keyCap = 0, K = 0;
    uint32_t chunk = 20, occupancy = 4, graphChunks = 8;
    uint32_t blockThreads = kFlatThreads;  // block size of the plain step kernels (64, 128, 256)
    bool anyPrecise = false, anyLocal = false;  // precision-form / cell-local mesh jobs
    bool anyPreciseCyl = false;                 // precision-form cylinder jobs
    bool anyLocalCyl = false;                   // cell-local cylinder jobs
    cudaGraphExec_t exec = nullptr;
    bool graphValid = false;
    int graphCur = -1;
    uint64_t launches = 0, graphLaunches = 0, bytes = 0;
};

namespace {

int balloc(dsim_batch* b, void** p, size_t bytes) {
    *p = nullptr;
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_last_error(kErrNoMem, "batch: cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
        return kErrNoMem;
    }
    b->bytes += bytes;
    return kOk;
}

BatchSpins view(dsim_batch* b, int which) {
    BatchSpins S;
    for (int f = 0; f < kBF; f++) S.f[f] = b->buf[which].f[f];
    for (int u = 0; u < kBU; u++) S.u[u] = b->buf[which].u[u];
    for (int f = 0; f < kBD; f++) S.d[f] = b->buf[which].d[f];
    S.N = (uint32_t)b->N;
    return S;
}

uint32_t sort_bits(uint32_t n) {
    // about two spins per sort cell: 2^(3 bits) ~ n / 2, 3..7 bits per axis
    uint32_t bits = 3;
    while (bits < 7 && (1ull << (3 * (bits + 1))) <= (uint64_t)n / 2) bits++;
    return bits;
}

void invalidate_graph(dsim_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    b->graphValid = false;
}

// recompute sort key bases in packing order and grow the histogram
int layout_keys(dsim_batch* b) {
    uint64_t K = 0, slot = 0;
    for (auto& j : b->jobs) {
        j.d.sortBase = (uint32_t)K;
        K += (j.d.sortRegion ? 2ull : 1ull) << (3 * j.d.sortBits);
        j.slot0 = slot;
        slot += j.pad;
    }
    if (K > 0xFFFFFFF0ull) { set_last_error(kErrTooLarge, "batch: sort key space too large"); return kErrTooLarge; }
    if (K > b->keyCap) {
        cudaFree(b->hist); cudaFree(b->hstart); cudaFree(b->scratch);
        b->hist = b->hstart = b->scratch = nullptr;
        uint64_t cap = std::max<uint64_t>(K, 1u << 16) * 2;
        int rc;
        if ((rc = balloc(b, (void**)&b->hist, cap * 4)) || (rc = balloc(b, (void**)&b->hstart, (cap + 1) * 4)) ||
            (rc = balloc(b, (void**)&b->scratch, scan_scratch_words((uint32_t)cap) * 4)))
            return rc;
        b->keyCap = cap;
    }
    b->K = K;
    return kOk;
}

int upload_jobs(dsim_batch* b) {
    std::vector<JobDev> h(b->jobs.size());
    for (size_t k = 0; k < b->jobs.size(); k++) h[k] = b->jobs[k].d;
    if (!h.empty()) DSIM_CUDA_TRY(cudaMemcpyAsync(b->d_jobs, h.data(), h.size() * sizeof(JobDev), cudaMemcpyHostToDevice, b->st));
    return kOk;
}

// which plain step instantiations a chunk launches: bit 1 / 2 for mesh jobs
// on 32- / 64-byte fine-grid records, bit 3 for cylinder jobs; bits 5 / 6 for
// cell-local mesh jobs on 32- / 64-byte records
uint32_t step_layouts(const dsim_batch* b) {
    uint32_t mask = 0;
    for (const auto& j : b->jobs) {
        const SubDev& s = b->subs[j.d.sub];
        if (s.kind == kSubCyl) { if (!j.d.flags) mask |= 1u << 3; }
        else if (!j.d.flags) mask |= 1u << (s.acc.wide == 2 ? 2u : 1u);
        else if (j.d.flags & DSIM_JOB_LOCAL) mask |= 1u << (s.acc.wide == 2 ? 6u : 5u);
    }
    return mask;
}

// kernels one chunk launches: keys, scan (3), scatter, the step
// instantiations, advance
uint64_t chunk_launches(const dsim_batch* b) {
    const uint32_t mask = step_layouts(b);
    return 5ull + (uint64_t)__builtin_popcount(mask & 0x6Eu) + (b->anyPrecise ? 1ull : 0ull) +
           (b->anyPreciseCyl ? 1ull : 0ull) + (b->anyLocalCyl ? 1ull : 0ull) + 1ull;
}

// Precision-form cylinder jobs (DSIM_JOB_PRECISE): the dSim2 step of
// cpuIntegrate (dSim2/src/spinKernelCpu.cpp:312-641) with positions,
// distances, clamp, T2 decay and moments in double (cyl_membranes64); the
// parameters are the job's float values.  Position and magnitude persist in
// the double fields; the moment is kept as the float pair m - c.
__global__ void __launch_bounds__(kFlatThreads, 4)
k_batch_step_cyl64(const SubDev* __restrict__ subs, const JobDev* __restrict__ jobs, BatchSpins S,
                   const uint32_t* __restrict__ stepNow, uint32_t chunk, uint32_t* status,
                   unsigned long long* jobCounts) {
    const uint32_t FULL = 0xFFFFFFFFu;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if ((i & ~31u) >= S.N) return;  // whole warp: N is a multiple of 32
    const uint32_t jb = S.u[U_JOB][i & ~31u];
    const JobDev& J = jobs[jb];
    if (!(__ldg(&J.flags) & DSIM_JOB_PRECISE)) return;  // warp-uniform
    const SubDev& sub = subs[__ldg(&J.sub)];
    if (__ldg(&sub.kind) != kSubCyl) return;
    const uint32_t now = *stepNow;
    const uint32_t start = __ldg(&J.start), steps = __ldg(&J.steps);
    if (now < start || now - start >= steps) return;
    const uint32_t ls0 = now - start;
    const uint32_t nsteps = min(chunk, steps - ls0);
    const uint32_t id = S.u[U_ID][i];
    const bool valid = id != 0xFFFFFFFFu;
    uint32_t nrefl = 0, nperm = 0, st = 0;
    if (valid) {
        const CylDev g = sub.c;
        double x = S.d[D_X][i], y = S.d[D_Y][i], z = S.d[D_Z][i], mag = S.d[D_MAG][i];
        double Mx = (double)S.f[F_MX][i] - (double)S.f[F_CX][i];
        double My = (double)S.f[F_MY][i] - (double)S.f[F_CY][i];
        double Mz = (double)S.f[F_MZ][i] - (double)S.f[F_CZ][i];
        const uint32_t meta = S.u[U_META][i];
        uint32_t imo = meta & 0xFFu, nearest = meta >> 8;
        if (imo < 2 && nearest >= g.nF) imo = 2;
        const double perm = (double)__ldg(&J.perm), inR = (double)__ldg(&J.inR);
        const double hiC = 1.0 - (double)__ldg(&J.spinR), loC = -1.0 + (double)__ldg(&J.spinR);
        const double dt = (double)__ldg(&J.dt);
        const uint32_t k0 = __ldg(&J.key0), k1 = __ldg(&J.key1);
        const float* __restrict__ wave = J.wave;
        for (uint32_t it = 0; it < nsteps; it++) {
            const Draw d = philox_draw(id, (uint64_t)(ls0 + it), 0u, k0, k1);
            const double ox = x, oy = y, oz = z;
            const double sd = (double)__ldg(&J.sd[imo == 0 ? 0 : (imo == 1 ? 1 : 2)]);
            double px = x + (double)d.nx * sd, py = y + (double)d.ny * sd, pz = z + (double)d.nz * sd;
            cyl_membranes64(g, ox, oy, oz, px, py, pz, (double)d.u, perm, inR, imo, nearest, nrefl, nperm, st);
            if (px > hiC) px = hiC; else if (px < loC) px = loC;
            if (py > hiC) py = hiC; else if (py < loC) py = loC;
            if (pz > hiC) pz = hiC; else if (pz < loC) pz = loC;
            x = px; y = py; z = pz;
            if (imo <= 2) {
                const float T2 = __ldg(&J.T2[imo]);
                if (T2 > 0.0f) mag += -mag / (double)T2 * dt;
            }
            const double w = (double)__ldg(wave + ls0 + it);
            Mx += w * x; My += w * y; Mz += w * z;
        }
        S.d[D_X][i] = x; S.d[D_Y][i] = y; S.d[D_Z][i] = z; S.d[D_MAG][i] = mag;
        S.f[F_X][i] = (float)x; S.f[F_Y][i] = (float)y; S.f[F_Z][i] = (float)z;
        S.f[F_MAG][i] = (float)mag;
        const float mx = (float)Mx, my = (float)My, mz = (float)Mz;
        S.f[F_MX][i] = mx; S.f[F_MY][i] = my; S.f[F_MZ][i] = mz;
        S.f[F_CX][i] = (float)((double)mx - Mx);
        S.f[F_CY][i] = (float)((double)my - My);
        S.f[F_CZ][i] = (float)((double)mz - Mz);
        S.u[U_META][i] = (imo & 0xFFu) | ((nearest & 0xFFFFFFu) << 8);
    }
    unsigned long long r = nrefl, p = nperm;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        r += __shfl_down_sync(FULL, r, o);
        p += __shfl_down_sync(FULL, p, o);
    }
    if (lane == 0) {
        if (r) atomicAdd(jobCounts + 4 * jb, r);
        if (p) atomicAdd(jobCounts + 4 * jb + 1, p);
    }
    if (st) atomicOr(status, st);
}

// Cell-local FP32 cylinder jobs (DSIM_JOB_LOCAL): the dSim2 step with the
// position as a lattice origin (multiple of 1/16) plus an FP32 offset in
// [0, 1/16), membrane decisions near their FP32 error band taken in FP64
// (cyl_membranes_local), Kahan moments.  Between chunks the position is kept
// in the double fields as origin + offset.
__global__ void __launch_bounds__(kFlatThreads, 4)
k_batch_step_cyl_local(const SubDev* __restrict__ subs, const JobDev* __restrict__ jobs, BatchSpins S,
                       const uint32_t* __restrict__ stepNow, uint32_t chunk, uint32_t* status,
                       unsigned long long* jobCounts) {
    __shared__ float mom[6][kFlatThreads];
    const uint32_t FULL = 0xFFFFFFFFu;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t tx = threadIdx.x;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if ((i & ~31u) >= S.N) return;  // whole warp: N is a multiple of 32
    const uint32_t jb = S.u[U_JOB][i & ~31u];
    const JobDev& J = jobs[jb];
    if (!(__ldg(&J.flags) & DSIM_JOB_LOCAL)) return;  // warp-uniform
    const SubDev& sub = subs[__ldg(&J.sub)];
    if (__ldg(&sub.kind) != kSubCyl) return;
    const uint32_t now = *stepNow;
    const uint32_t start = __ldg(&J.start), steps = __ldg(&J.steps);
    if (now < start || now - start >= steps) return;
    const uint32_t ls0 = now - start;
    const uint32_t nsteps = min(chunk, steps - ls0);
    const uint32_t id = S.u[U_ID][i];
    const bool valid = id != 0xFFFFFFFFu;
    uint32_t nrefl = 0, nperm = 0, st = 0, ntests = 0, nexact = 0;
    if (valid) {
        const CylDev g = sub.c;
        const double X = S.d[D_X][i], Y = S.d[D_Y][i], Z = S.d[D_Z][i];
        CylOrigin G;
        G.x = (float)(floor(X * 16.0) * 0.0625);
        G.y = (float)(floor(Y * 16.0) * 0.0625);
        G.z = (float)(floor(Z * 16.0) * 0.0625);
        float x = (float)(X - (double)G.x), y = (float)(Y - (double)G.y), z = (float)(Z - (double)G.z);
        float mag = S.f[F_MAG][i];
        mom[0][tx] = S.f[F_MX][i]; mom[1][tx] = S.f[F_MY][i]; mom[2][tx] = S.f[F_MZ][i];
        mom[3][tx] = S.f[F_CX][i]; mom[4][tx] = S.f[F_CY][i]; mom[5][tx] = S.f[F_CZ][i];
        const uint32_t meta = S.u[U_META][i];
        uint32_t imo = meta & 0xFFu, nearest = meta >> 8;
        if (imo < 2 && nearest >= g.nF) imo = 2;
        const float perm = __ldg(&J.perm), inR = __ldg(&J.inR);
        const float clampHi = __ldg(&J.clampHi), clampLo = __ldg(&J.clampLo), dt = __ldg(&J.dt);
        const uint32_t k0 = __ldg(&J.key0), k1 = __ldg(&J.key1);
        const float* __restrict__ wave = J.wave;
        for (uint32_t it = 0; it < nsteps; it++) {
            const Draw d = philox_draw(id, (uint64_t)(ls0 + it), 0u, k0, k1);
            const float ox = x, oy = y, oz = z;
            const float sd = __ldg(&J.sd[imo < 3 ? imo : 2]);
            float px = x + d.nx * sd, py = y + d.ny * sd, pz = z + d.nz * sd;
            cyl_membranes_local(g, G, ox, oy, oz, px, py, pz, d.u, perm, inR, imo, nearest, nrefl, nperm, st, ntests,
                                nexact);
            // clamp in absolute coordinates, then move the origin so the
            // offset is back in [0, 1/16)
            if (G.x + px > clampHi) px = clampHi - G.x; else if (G.x + px < clampLo) px = clampLo - G.x;
            if (G.y + py > clampHi) py = clampHi - G.y; else if (G.y + py < clampLo) py = clampLo - G.y;
            if (G.z + pz > clampHi) pz = clampHi - G.z; else if (G.z + pz < clampLo) pz = clampLo - G.z;
            const float sx = floor_small(px * 16.0f) * kLatticeH, sy = floor_small(py * 16.0f) * kLatticeH,
                        sz = floor_small(pz * 16.0f) * kLatticeH;
            G.x += sx; G.y += sy; G.z += sz;
            x = px - sx; y = py - sy; z = pz - sz;
            const float T2 = __ldg(&J.T2[imo < 3 ? imo : 2]);
            if (T2 > 0.0f) mag += -mag / T2 * dt;
            const float w = __ldg(wave + ls0 + it);
            kahan_add(mom[0][tx], mom[3][tx], w * (G.x + x));
            kahan_add(mom[1][tx], mom[4][tx], w * (G.y + y));
            kahan_add(mom[2][tx], mom[5][tx], w * (G.z + z));
        }
        const double Xn = (double)G.x + (double)x, Yn = (double)G.y + (double)y, Zn = (double)G.z + (double)z;
        S.d[D_X][i] = Xn; S.d[D_Y][i] = Yn; S.d[D_Z][i] = Zn; S.d[D_MAG][i] = (double)mag;
        S.f[F_X][i] = (float)Xn; S.f[F_Y][i] = (float)Yn; S.f[F_Z][i] = (float)Zn;
        S.f[F_MAG][i] = mag;
        S.f[F_MX][i] = mom[0][tx]; S.f[F_MY][i] = mom[1][tx]; S.f[F_MZ][i] = mom[2][tx];
        S.f[F_CX][i] = mom[3][tx]; S.f[F_CY][i] = mom[4][tx]; S.f[F_CZ][i] = mom[5][tx];
        S.u[U_META][i] = (imo & 0xFFu) | ((nearest & 0xFFFFFFu) << 8);
    }
    // per-job counters {reflections, permeations, distance tests, FP64 decisions}
    unsigned long long r = nrefl, p = nperm, te = ntests, ex = nexact;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        r += __shfl_down_sync(FULL, r, o);
        p += __shfl_down_sync(FULL, p, o);
        te += __shfl_down_sync(FULL, te, o);
        ex += __shfl_down_sync(FULL, ex, o);
    }
    if (lane == 0) {
        if (r) atomicAdd(jobCounts + 4 * jb, r);
        if (p) atomicAdd(jobCounts + 4 * jb + 1, p);
        if (te) atomicAdd(jobCounts + 4 * jb + 2, te);
        if (ex) atomicAdd(jobCounts + 4 * jb + 3, ex);
    }
    if (st) atomicOr(status, st);
}

template <int LAYOUT, int THREADS>
void launch_step_shape(dsim_batch* b, const BatchSpins& D, cudaStream_t st) {
    const uint32_t grid = (uint32_t)((b->N + THREADS - 1) / THREADS);
    if (b->occupancy >= 8)
        k_batch_step<8, LAYOUT, THREADS><<<grid, THREADS, 0, st>>>(b->d_subs, b->d_jobs, D, b->d_stepNow, b->chunk,
                                                                  b->d_status, b->d_counts);
    else if (b->occupancy >= 6)
        k_batch_step<6, LAYOUT, THREADS><<<grid, THREADS, 0, st>>>(b->d_subs, b->d_jobs, D, b->d_stepNow, b->chunk,
                                                                  b->d_status, b->d_counts);
    else if (b->occupancy == 5)
        k_batch_step<5, LAYOUT, THREADS><<<grid, THREADS, 0, st>>>(b->d_subs, b->d_jobs, D, b->d_stepNow, b->chunk,
                                                                  b->d_status, b->d_counts);
    else
        k_batch_step<4, LAYOUT, THREADS><<<grid, THREADS, 0, st>>>(b->d_subs, b->d_jobs, D, b->d_stepNow, b->chunk,
                                                                  b->d_status, b->d_counts);
}

template <int LAYOUT>
void launch_step_layout(dsim_batch* b, const BatchSpins& D, cudaStream_t st) {
    if (b->blockThreads == 64) launch_step_shape<LAYOUT, 64>(b, D, st);
    else if (b->blockThreads == 256) launch_step_shape<LAYOUT, 256>(b, D, st);
    else launch_step_shape<LAYOUT, kFlatThreads>(b, D, st);
}

// one chunk: sort into the other buffer, step, advance the step counter
int enqueue_chunk(dsim_batch* b) {
    const uint32_t N = (uint32_t)b->N;
    const uint32_t nb = (N + 255) / 256;
    BatchSpins S = view(b, b->cur), D = view(b, 1 - b->cur);
    DSIM_CUDA_TRY(cudaMemsetAsync(b->hist, 0, b->K * 4, b->st));
    k_batch_keys<<<nb, 256, 0, b->st>>>(b->d_jobs, S, b->keys, b->hist);
    int rc = launch_scan_exclusive(b->hist, b->hstart, (uint32_t)b->K, b->scratch, b->st);
    if (rc) return rc;
    DSIM_CUDA_TRY(cudaMemsetAsync(b->hist, 0, b->K * 4, b->st));
    k_batch_scatter<<<nb, 256, 0, b->st>>>(S, D, b->keys, b->hstart, b->hist);
    b->cur = 1 - b->cur;
    const uint32_t grid = (N + kFlatThreads - 1) / kFlatThreads;
    const uint32_t mask = step_layouts(b);
    // the step kernels this chunk needs, each on its own stream when there
    // are several (they advance disjoint jobs)
    int kinds[8], nk = 0;
    for (int L = 1; L <= 3; L++)
        if (mask & (1u << L)) kinds[nk++] = L;
    for (int L = 5; L <= 6; L++)
        if (mask & (1u << L)) kinds[nk++] = 4 + 4 * (L - 5);  // 4, 8: cell-local mesh, 32- / 64-byte records
    if (b->anyPrecise) kinds[nk++] = 5;
    if (b->anyPreciseCyl) kinds[nk++] = 6;
    if (b->anyLocalCyl) kinds[nk++] = 7;
    const bool fork = nk > 1;
    if (fork) DSIM_CUDA_TRY(cudaEventRecord(b->forkEv, b->st));
    for (int q = 0; q < nk; q++) {
        cudaStream_t st = fork ? b->side[q % dsim_batch::kSide] : b->st;
        if (fork) DSIM_CUDA_TRY(cudaStreamWaitEvent(st, b->forkEv, 0));
        switch (kinds[q]) {
            case 1: launch_step_layout<1>(b, D, st); break;
            case 2: launch_step_layout<2>(b, D, st); break;
            case 3: launch_step_layout<3>(b, D, st); break;
            case 4:
                k_batch_step_local<1><<<grid, kFlatThreads, 0, st>>>(b->d_subs, b->d_jobs, D, b->d_stepNow,
                                                                     b->chunk, b->d_status, b->d_counts);
                break;
            case 8:
                k_batch_step_local<2><<<grid, kFlatThreads, 0, st>>>(b->d_subs, b->d_jobs, D, b->d_stepNow,
                                                                     b->chunk, b->d_status, b->d_counts);
                break;
            case 5:
                k_batch_step64<<<grid, kFlatThreads, 0, st>>>(b->d_subs, b->d_jobs, D, b->d_stepNow, b->chunk,
                                                              b->d_status, b->d_counts);
                break;
            case 6:
                k_batch_step_cyl64<<<grid, kFlatThreads, 0, st>>>(b->d_subs, b->d_jobs, D, b->d_stepNow, b->chunk,
                                                                  b->d_status, b->d_counts);
                break;
            default:
                k_batch_step_cyl_local<<<grid, kFlatThreads, 0, st>>>(b->d_subs, b->d_jobs, D, b->d_stepNow,
                                                                      b->chunk, b->d_status, b->d_counts);
                break;
        }
        if (fork) {
            DSIM_CUDA_TRY(cudaEventRecord(b->joinEv[q % dsim_batch::kSide], st));
            DSIM_CUDA_TRY(cudaStreamWaitEvent(b->st, b->joinEv[q % dsim_batch::kSide], 0));
        }
    }
    k_batch_advance<<<1, 1, 0, b->st>>>(b->d_stepNow, b->chunk);
    DSIM_CUDA_TRY(cudaGetLastError());
    b->launches += chunk_launches(b);  // keys, scan (3), scatter, step (per layout), advance
    return kOk;
}

int capture_graph(dsim_batch* b) {
    invalidate_graph(b);
    const uint32_t G = b->graphChunks & ~1u;  // even: the buffers end where they start
    if (G == 0) return kOk;
    const int cur0 = b->cur;
    const uint64_t launches0 = b->launches;
    cudaGraph_t graph = nullptr;
    DSIM_CUDA_TRY(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
    int rc = kOk;
    for (uint32_t c = 0; c < G && !rc; c++) rc = enqueue_chunk(b);
    cudaError_t e = cudaStreamEndCapture(b->st, &graph);
    b->cur = cur0;
    b->launches = launches0;
    if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
    if (e != cudaSuccess) { set_last_cuda_error(e, "cudaStreamEndCapture", __FILE__, __LINE__); return kErrCuda; }
    e = cudaGraphInstantiate(&b->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) { b->exec = nullptr; set_last_cuda_error(e, "cudaGraphInstantiate", __FILE__, __LINE__); return kErrCuda; }
    b->graphValid = true;
    b->graphCur = cur0;
    return kOk;
}

bool job_finished(const dsim_batch* b, const BatchJob& j) {
    return b->stepNow >= j.d.start && b->stepNow - j.d.start >= j.d.steps;
}

BatchJob* find_job(dsim_batch* b, uint32_t id) {
    for (auto& j : b->jobs)
        if (j.id == id) return &j;
    return nullptr;
}

constexpr double kPi = 3.14159265358979323846;

std::vector<float> make_wave(const dsim_job_desc* d) {
    std::vector<float> w(d->steps, 0.0f);
    if (d->waveform == DSIM_WAVE_TABLE) {
        for (uint32_t s = 0; s < d->steps; s++) w[s] = d->table[s];
        return w;
    }
    const long nd = lround((double)d->delta / (double)d->deltaTime);
    const long nD = lround((double)d->Delta / (double)d->deltaTime);
    for (uint32_t s = 0; s < d->steps; s++) {
        const long t = (long)s;
        if (t < nd) {
            w[s] = d->waveform == DSIM_WAVE_OGSE
                       ? (float)std::cos(2.0 * kPi * (double)d->frequency * 1e-3 * (double)t * (double)d->deltaTime)
                       : 1.0f;
        } else if (t >= nD && t < nD + nd) {
            w[s] = d->waveform == DSIM_WAVE_OGSE
                       ? -(float)std::cos(2.0 * kPi * (double)d->frequency * 1e-3 * (double)(t - nD) * (double)d->deltaTime)
                       : -1.0f;
        }
    }
    return w;
}

}  // namespace

extern "C" {

int dsim_batch_create(uint64_t spinCapacity, uint32_t jobCapacity, dsim_batch** out) {
    if (!out || spinCapacity == 0 || jobCapacity == 0 || spinCapacity > 0xFFFFFFE0ull) {
        set_last_error(kErrInvalid, "dsim_batch_create: bad argument");
        return kErrInvalid;
    }
    *out = nullptr;
    dsim_batch* b = new dsim_batch();
    b->cap = (spinCapacity + 31) & ~31ull;
    b->jobCap = jobCapacity;
    int rc = kOk;
    if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess) rc = kErrCuda;
    for (int k = 0; k < dsim_batch::kSide && !rc; k++)
        if (cudaStreamCreateWithFlags(&b->side[k], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->joinEv[k], cudaEventDisableTiming) != cudaSuccess)
            rc = kErrCuda;
    if (!rc && cudaEventCreateWithFlags(&b->forkEv, cudaEventDisableTiming) != cudaSuccess) rc = kErrCuda;
    for (int k = 0; k < 2 && !rc; k++) {
        for (int f = 0; f < kBF && !rc; f++) rc = balloc(b, (void**)&b->buf[k].f[f], b->cap * 4);
        for (int u = 0; u < kBU && !rc; u++) rc = balloc(b, (void**)&b->buf[k].u[u], b->cap * 4);
    }
    if (!rc) rc = balloc(b, (void**)&b->keys, b->cap * 4);
    if (!rc) rc = balloc(b, (void**)&b->d_jobs, (size_t)jobCapacity * sizeof(JobDev));
    if (!rc) rc = balloc(b, (void**)&b->d_subs, (size_t)b->subCap * sizeof(SubDev));
    if (!rc) rc = balloc(b, (void**)&b->d_counts, (size_t)4 * jobCapacity * 8);
    if (!rc) rc = balloc(b, (void**)&b->d_status, 4);
    if (!rc) rc = balloc(b, (void**)&b->d_stepNow, 4);
    if (!rc && (cudaMemset(b->d_status, 0, 4) != cudaSuccess || cudaMemset(b->d_stepNow, 0, 4) != cudaSuccess ||
                cudaMemset(b->d_counts, 0, (size_t)4 * jobCapacity * 8) != cudaSuccess))
        rc = kErrCuda;
    if (rc) { dsim_batch_free(b); return rc; }
    *out = b;
    return kOk;
}

void dsim_batch_free(dsim_batch* b) {
    if (!b) return;
    if (b->st) cudaStreamSynchronize(b->st);
    invalidate_graph(b);
    for (int k = 0; k < 2; k++) {
        for (int f = 0; f < kBF; f++) cudaFree(b->buf[k].f[f]);
        for (int u = 0; u < kBU; u++) cudaFree(b->buf[k].u[u]);
        for (int f = 0; f < kBD; f++) cudaFree(b->buf[k].d[f]);
    }
    for (auto& j : b->jobs) cudaFree(j.wave);
    cudaFree(b->keys); cudaFree(b->hist); cudaFree(b->hstart); cudaFree(b->scratch);
    cudaFree(b->d_jobs); cudaFree(b->d_subs); cudaFree(b->d_counts); cudaFree(b->d_status);
    cudaFree(b->d_stepNow);
    if (b->st) cudaStreamDestroy(b->st);
    for (int k = 0; k < dsim_batch::kSide; k++) {
        if (b->side[k]) cudaStreamDestroy(b->side[k]);
        if (b->joinEv[k]) cudaEventDestroy(b->joinEv[k]);
    }
    if (b->forkEv) cudaEventDestroy(b->forkEv);
    for (const dsim_cyl* c : b->cylsHeld) cyl_hold(c, -1);
    delete b;
}

static int add_sub(dsim_batch* b, const SubDev& s, const dsim_mesh* m, uint32_t* id) {
    if (b->subs.size() >= b->subCap) { set_last_error(kErrTooLarge, "batch: too many substrates"); return kErrTooLarge; }
    b->subs.push_back(s);
    b->meshes.push_back(m);
    DSIM_CUDA_TRY(cudaMemcpyAsync(b->d_subs + (b->subs.size() - 1), &s, sizeof(SubDev), cudaMemcpyHostToDevice, b->st));
    DSIM_CUDA_TRY(cudaStreamSynchronize(b->st));
    *id = (uint32_t)(b->subs.size() - 1);
    return kOk;
}

int dsim_batch_add_mesh(dsim_batch* b, const dsim_mesh* m, uint32_t* substrate) {
    if (!b || !m || !substrate) { set_last_error(kErrInvalid, "dsim_batch_add_mesh: null argument"); return kErrInvalid; }
    SubDev s;
    memset(&s, 0, sizeof(s));
    s.kind = kSubMesh;
    int rc = mesh_views(m, &s.g, &s.acc);
    if (rc) return rc;
    return add_sub(b, s, m, substrate);
}

int dsim_batch_add_cyl(dsim_batch* b, const dsim_cyl* c, uint32_t* substrate) {
    if (!b || !c || !substrate) { set_last_error(kErrInvalid, "dsim_batch_add_cyl: null argument"); return kErrInvalid; }
    SubDev s;
    memset(&s, 0, sizeof(s));
    s.kind = kSubCyl;
    int rc = cyl_view(c, &s.c);
    if (rc) return rc;
    if ((rc = add_sub(b, s, nullptr, substrate))) return rc;
    cyl_hold(c, 1);
    b->cylsHeld.push_back(c);
    return kOk;
}

// first precision-form job on a substrate: the mesh's FP64 triangle table, and
// for the batch the FP64 state fields of both spin buffers
static int ensure_precise(dsim_batch* b, uint32_t substrate) {
    int rc = kOk;
    SubDev& sd = b->subs[substrate];
    if (sd.kind == kSubMesh) {
        dsim_mesh* m = const_cast<dsim_mesh*>(b->meshes[substrate]);
        if ((rc = mesh_tri64(m))) return rc;
    }
    if (sd.kind == kSubMesh && !sd.g.tri64) {
        dsim_mesh* m = const_cast<dsim_mesh*>(b->meshes[substrate]);
        if ((rc = mesh_views(m, &sd.g, &sd.acc))) return rc;
        DSIM_CUDA_TRY(cudaMemcpyAsync(b->d_subs + substrate, &sd, sizeof(SubDev), cudaMemcpyHostToDevice, b->st));
        invalidate_graph(b);
    }
    if (!b->buf[0].d[0]) {
        for (int k = 0; k < 2; k++)
            for (int f = 0; f < kBD; f++)
                if ((rc = balloc(b, (void**)&b->buf[k].d[f], b->cap * 8))) return rc;
        invalidate_graph(b);
    }
    return kOk;
}

int dsim_batch_submit(dsim_batch* b, const dsim_job_desc* d, const float* pos3, const uint8_t* comp,
                      const uint32_t* fiber, uint32_t* jobId) {
    if (!b || !d || !pos3 || !comp || !jobId || d->nSpins == 0 || d->steps == 0 || d->substrate >= b->subs.size() ||
        !(d->deltaTime > 0.0f) || (d->waveform == DSIM_WAVE_TABLE && !d->table) || d->waveform > DSIM_WAVE_TABLE) {
        set_last_error(kErrInvalid, "dsim_batch_submit: bad argument");
        return kErrInvalid;
    }
    const uint32_t pad = (d->nSpins + 31u) & ~31u;
    if (b->N + pad > b->cap || b->jobs.size() >= b->jobCap) {
        set_last_error(kErrNoMem, "dsim_batch_submit: batch full (%llu + %u spins of %llu, %zu jobs of %u)",
                       (unsigned long long)b->N, pad, (unsigned long long)b->cap, b->jobs.size(), b->jobCap);
        return kErrNoMem;
    }
    const bool cyl = b->subs[d->substrate].kind == kSubCyl;
    BatchJob j;
    j.id = b->nextId;
    j.nSpins = d->nSpins;
    j.pad = pad;
    j.pc = (double)d->phaseConstant;
    JobDev& J = j.d;
    memset(&J, 0, sizeof(J));
    J.sub = d->substrate;
    J.steps = d->steps;
    J.start = b->stepNow;
    J.sortBits = sort_bits(d->nSpins);
    J.sortRegion = cyl ? 1u : 0u;
    for (int k = 0; k < 4; k++) { J.sd[k] = d->stepSd[k]; J.T2[k] = d->T2[k]; }
    J.perm = d->permeability;
    J.dt = d->deltaTime;
    J.clampHi = 1.0f - d->spinRadius;
    J.clampLo = -1.0f + d->spinRadius;
    J.reflType = d->reflectionType;
    J.maxSub = 4096;
    J.inR = d->innerRadiusProportion * d->innerRadiusProportion;
    J.key0 = (uint32_t)d->seed;
    J.key1 = (uint32_t)(d->seed >> 32);
    J.flags = d->flags & (DSIM_JOB_PRECISE | DSIM_JOB_LOCAL);
    if (J.flags == (DSIM_JOB_PRECISE | DSIM_JOB_LOCAL)) {
        set_last_error(kErrInvalid, "dsim_batch_submit: DSIM_JOB_PRECISE and DSIM_JOB_LOCAL exclude each other");
        return kErrInvalid;
    }
    J.spinR = d->spinRadius;
    if (J.flags) {
        int rc = ensure_precise(b, d->substrate);
        if (rc) return rc;
    }
    std::vector<float> w = make_wave(d);
    int rc = balloc(b, (void**)&j.wave, w.size() * 4);
    if (rc) return rc;
    J.wave = j.wave;
    if (!J.wave || w.size() < J.steps) {
        cudaFree(j.wave);
        set_last_error(kErrInvalid, "dsim_batch_submit: waveform table missing");
        return kErrInvalid;
    }
    if (cudaMemcpyAsync(j.wave, w.data(), w.size() * 4, cudaMemcpyHostToDevice, b->st) != cudaSuccess) {
        cudaFree(j.wave);
        set_last_error(kErrCuda, "dsim_batch_submit: waveform upload");
        return kErrCuda;
    }
    // host staging of the packed slots [N, N + pad)
    std::vector<float> hf[kBF];
    std::vector<uint32_t> hu[kBU];
    for (int f = 0; f < kBF; f++) hf[f].assign(pad, 0.0f);
    for (int u = 0; u < kBU; u++) hu[u].assign(pad, 0u);
    const uint32_t jobIndex = (uint32_t)b->jobs.size();
    for (uint32_t k = 0; k < pad; k++) {
        hu[U_JOB][k] = jobIndex;
        if (k < d->nSpins) {
            hf[F_X][k] = pos3[3 * k]; hf[F_Y][k] = pos3[3 * k + 1]; hf[F_Z][k] = pos3[3 * k + 2];
            hf[F_MAG][k] = 1.0f;
            uint32_t fb = fiber ? fiber[k] : 0xFFFFFFFFu;
            fb = cyl ? (fb & 0xFFFFFFu) : (fb & 0xFFFFu);
            hu[U_META][k] = (uint32_t)comp[k] | (fb << 8);
            hu[U_ID][k] = k;
        } else {
            hu[U_ID][k] = 0xFFFFFFFFu;
        }
    }
    for (int f = 0; f < kBF; f++)
        DSIM_CUDA_TRY(cudaMemcpyAsync(b->buf[b->cur].f[f] + b->N, hf[f].data(), (size_t)pad * 4, cudaMemcpyHostToDevice, b->st));
    for (int u = 0; u < kBU; u++)
        DSIM_CUDA_TRY(cudaMemcpyAsync(b->buf[b->cur].u[u] + b->N, hu[u].data(), (size_t)pad * 4, cudaMemcpyHostToDevice, b->st));
    if (J.flags) {
        // the FP64 state of the precision and cell-local forms: the given positions, magnitude 1
        std::vector<double> hd[kBD];
        for (int f = 0; f < kBD; f++) hd[f].assign(pad, 0.0);
        for (uint32_t k = 0; k < d->nSpins; k++) {
            hd[D_X][k] = pos3[3 * k]; hd[D_Y][k] = pos3[3 * k + 1]; hd[D_Z][k] = pos3[3 * k + 2];
            hd[D_MAG][k] = 1.0;
        }
        for (int f = 0; f < kBD; f++)
            DSIM_CUDA_TRY(cudaMemcpyAsync(b->buf[b->cur].d[f] + b->N, hd[f].data(), (size_t)pad * 8, cudaMemcpyHostToDevice, b->st));
        DSIM_CUDA_TRY(cudaStreamSynchronize(b->st));
    }
    b->jobs.push_back(j);
    b->nextId++;
    b->N += pad;
    if ((rc = layout_keys(b)) || (rc = upload_jobs(b))) return rc;
    DSIM_CUDA_TRY(cudaMemsetAsync(b->d_counts + 4 * jobIndex, 0, 32, b->st));
    DSIM_CUDA_TRY(cudaStreamSynchronize(b->st));
    if (J.flags & DSIM_JOB_PRECISE) (cyl ? b->anyPreciseCyl : b->anyPrecise) = true;
    if (J.flags & DSIM_JOB_LOCAL) (cyl ? b->anyLocalCyl : b->anyLocal) = true;
    invalidate_graph(b);
    *jobId = j.id;
    return kOk;
}

int dsim_batch_configure(dsim_batch* b, uint32_t chunk, uint32_t occupancy, uint32_t graphChunks) {
    if (!b || chunk == 0 || (occupancy != 4 && occupancy != 5 && occupancy != 6 && occupancy != 8)) {
        set_last_error(kErrInvalid, "dsim_batch_configure: chunk > 0, occupancy 4, 5, 6 or 8");
        return kErrInvalid;
    }
    b->chunk = chunk;
    b->occupancy = occupancy;
    b->graphChunks = graphChunks;
    invalidate_graph(b);
    return kOk;
}

int dsim_batch_block(const dsim_batch* b, uint32_t* threads) {
    if (!b || !threads) return kErrInvalid;
    *threads = b->blockThreads;
    return kOk;
}

int dsim_batch_set_block(dsim_batch* b, uint32_t threads) {
    if (!b || (threads != 64 && threads != 128 && threads != 256)) {
        set_last_error(kErrInvalid, "dsim_batch_set_block: 64, 128 or 256 threads");
        return kErrInvalid;
    }
    b->blockThreads = threads;
    invalidate_graph(b);
    return kOk;
}

static uint32_t remaining_steps(const dsim_batch* b) {
    uint32_t r = 0;
    for (const auto& j : b->jobs) {
        if (j.retired || job_finished(b, j)) continue;
        uint32_t left = j.d.steps - (b->stepNow - j.d.start);
        r = std::max(r, left);
    }
    return r;
}

int dsim_batch_advance(dsim_batch* b, uint32_t steps) {
    if (!b) return kErrInvalid;
    if (b->N == 0 || steps == 0) return kOk;
    uint32_t chunks = (steps + b->chunk - 1) / b->chunk;
    const uint32_t G = b->graphChunks & ~1u;
    while (chunks > 0) {
        if (G > 0 && chunks >= G) {
            if (!b->graphValid || b->graphCur != b->cur) {
                int rc = capture_graph(b);
                if (rc) return rc;
            }
            DSIM_CUDA_TRY(cudaGraphLaunch(b->exec, b->st));
            b->graphLaunches++;
            b->launches += chunk_launches(b) * G;
            b->stepNow += G * b->chunk;
            chunks -= G;
        } else {
            int rc = enqueue_chunk(b);
            if (rc) return rc;
            b->stepNow += b->chunk;
            chunks--;
        }
    }
    return kOk;
}

int dsim_batch_run(dsim_batch* b) {
    if (!b) return kErrInvalid;
    uint32_t left = remaining_steps(b);
    int rc = dsim_batch_advance(b, left);
    if (rc) return rc;
    DSIM_CUDA_TRY(cudaStreamSynchronize(b->st));
    return kOk;
}

int dsim_batch_job_status(dsim_batch* b, uint32_t jobId, uint32_t* stepsDone, int* done) {
    BatchJob* j = b ? find_job(b, jobId) : nullptr;
    if (!j) { set_last_error(kErrInvalid, "dsim_batch_job_status: unknown job %u", jobId); return kErrInvalid; }
    uint32_t s = b->stepNow >= j->d.start ? std::min(b->stepNow - j->d.start, j->d.steps) : 0u;
    if (stepsDone) *stepsDone = s;
    if (done) *done = s >= j->d.steps ? 1 : 0;
    return kOk;
}

int dsim_batch_signal(dsim_batch* b, uint32_t jobId, const float* gradScaled, uint32_t nG, double* out) {
    return dsim_batch_signal_region(b, jobId, gradScaled, nG, 0.0, out);
}

int dsim_batch_signal_region(dsim_batch* b, uint32_t jobId, const float* gradScaled, uint32_t nG, double region,
                             double* out) {
    BatchJob* j = b ? find_job(b, jobId) : nullptr;
    if (!j || !gradScaled || !out || nG == 0 || !(region >= 0.0)) {
        set_last_error(kErrInvalid, "dsim_batch_signal: bad argument");
        return kErrInvalid;
    }
    // warps: 32 gradients x one spin segment each, about 16 warps per SM in all
    const uint32_t gw = (nG + 31u) / 32u;
    const uint32_t nseg = std::max<uint32_t>(1u, std::min<uint32_t>((j->pad + 63u) / 64u, std::max<uint32_t>(1u, 2432u / gw)));
    const uint32_t segLen = (j->pad + nseg - 1u) / nseg;
    const uint32_t nb = nseg;  // partial records per gradient
    std::vector<double> kg(3 * (size_t)nG);
    // phase = phaseConstant * (g . M); the job keeps phaseConstant in its descriptor
    for (uint32_t g = 0; g < nG; g++)
        for (int c = 0; c < 3; c++) kg[3 * g + c] = j->pc * (double)gradScaled[3 * g + c];
    double *dk = nullptr, *dp = nullptr, *dout = nullptr;
    int rc;
    if ((rc = balloc(b, (void**)&dk, kg.size() * 8)) || (rc = balloc(b, (void**)&dp, (size_t)nb * nG * 15 * 8)) ||
        (rc = balloc(b, (void**)&dout, (size_t)nG * 15 * 8))) {
        cudaFree(dk); cudaFree(dp); cudaFree(dout);
        return rc;
    }
    b->bytes -= kg.size() * 8 + (size_t)nb * nG * 15 * 8 + (size_t)nG * 15 * 8;
    cudaError_t e = cudaMemcpyAsync(dk, kg.data(), kg.size() * 8, cudaMemcpyHostToDevice, b->st);
    if (e == cudaSuccess) {
        const uint32_t warps = gw * nseg;
        k_batch_signal<<<(warps * 32u + kSigThreads - 1) / kSigThreads, kSigThreads, 0, b->st>>>(
            view(b, b->cur), (uint32_t)j->slot0, j->pad, dk, nG, gw, nseg, segLen, region,
            j->d.flags != 0 && b->buf[b->cur].d[0] != nullptr, dp);
        k_batch_signal_final<<<(nG * 15 + 127) / 128, 128, 0, b->st>>>(dp, nb, nG, dout);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, (size_t)nG * 15 * 8, cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    cudaFree(dk); cudaFree(dp); cudaFree(dout);
    if (e != cudaSuccess) { set_last_cuda_error(e, "dsim_batch_signal", __FILE__, __LINE__); return kErrCuda; }
    return kOk;
}

int dsim_batch_get(dsim_batch* b, uint32_t jobId, float* pos3, float* mag, float* moments6, uint8_t* compartment,
                   uint32_t* fiber) {
    BatchJob* j = b ? find_job(b, jobId) : nullptr;
    if (!j) { set_last_error(kErrInvalid, "dsim_batch_get: unknown job %u", jobId); return kErrInvalid; }
    const uint32_t n = j->nSpins;
    float *dp = nullptr, *dm = nullptr, *dmo = nullptr;
    uint32_t* dme = nullptr;
    int rc;
    if ((rc = balloc(b, (void**)&dp, (size_t)n * 12)) || (rc = balloc(b, (void**)&dm, (size_t)n * 4)) ||
        (rc = balloc(b, (void**)&dmo, (size_t)n * 24)) || (rc = balloc(b, (void**)&dme, (size_t)n * 4))) {
        cudaFree(dp); cudaFree(dm); cudaFree(dmo); cudaFree(dme);
        return rc;
    }
    b->bytes -= (size_t)n * 44;
    k_batch_gather<<<(j->pad + 255) / 256, 256, 0, b->st>>>(view(b, b->cur), (uint32_t)j->slot0, j->pad, dp, dm, dmo, dme);
    cudaError_t e = cudaGetLastError();
    std::vector<float> hp(3 * (size_t)n), hm(n), hmo(6 * (size_t)n);
    std::vector<uint32_t> hme(n);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hp.data(), dp, (size_t)n * 12, cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hm.data(), dm, (size_t)n * 4, cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hmo.data(), dmo, (size_t)n * 24, cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hme.data(), dme, (size_t)n * 4, cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    cudaFree(dp); cudaFree(dm); cudaFree(dmo); cudaFree(dme);
    if (e != cudaSuccess) { set_last_cuda_error(e, "dsim_batch_get", __FILE__, __LINE__); return kErrCuda; }
    if (pos3) memcpy(pos3, hp.data(), hp.size() * 4);
    if (mag) memcpy(mag, hm.data(), hm.size() * 4);
    if (moments6) memcpy(moments6, hmo.data(), hmo.size() * 4);
    for (uint32_t k = 0; k < n; k++) {
        if (compartment) compartment[k] = (uint8_t)(hme[k] & 0xFFu);
        if (fiber) fiber[k] = hme[k] >> 8;
    }
    return kOk;
}

int dsim_batch_get_precise(dsim_batch* b, uint32_t jobId, double* pos3, double* mag) {
    BatchJob* j = b ? find_job(b, jobId) : nullptr;
    if (!j || !j->d.flags) {
        set_last_error(kErrInvalid, "dsim_batch_get_precise: %u is neither a precision-form nor a cell-local job", jobId);
        return kErrInvalid;
    }
    const uint32_t n = j->nSpins;
    double *dp = nullptr, *dm = nullptr;
    int rc;
    if ((rc = balloc(b, (void**)&dp, (size_t)n * 24)) || (rc = balloc(b, (void**)&dm, (size_t)n * 8))) {
        cudaFree(dp); cudaFree(dm);
        return rc;
    }
    b->bytes -= (size_t)n * 32;
    k_batch_gather64<<<(j->pad + 255) / 256, 256, 0, b->st>>>(view(b, b->cur), (uint32_t)j->slot0, j->pad, dp, dm);
    cudaError_t e = cudaGetLastError();
    std::vector<double> hp(3 * (size_t)n), hm(n);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hp.data(), dp, (size_t)n * 24, cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hm.data(), dm, (size_t)n * 8, cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    cudaFree(dp); cudaFree(dm);
    if (e != cudaSuccess) { set_last_cuda_error(e, "dsim_batch_get_precise", __FILE__, __LINE__); return kErrCuda; }
    if (pos3) memcpy(pos3, hp.data(), hp.size() * 8);
    if (mag) memcpy(mag, hm.data(), hm.size() * 8);
    return kOk;
}

int dsim_batch_counts(dsim_batch* b, uint32_t jobId, uint64_t counts[2]) {
    if (!b || !counts) return kErrInvalid;
    for (size_t k = 0; k < b->jobs.size(); k++) {
        if (b->jobs[k].id != jobId) continue;
        unsigned long long c[4];
        DSIM_CUDA_TRY(cudaMemcpyAsync(c, b->d_counts + 4 * k, 32, cudaMemcpyDeviceToHost, b->st));
        DSIM_CUDA_TRY(cudaStreamSynchronize(b->st));
        counts[0] = c[0]; counts[1] = c[1];
        return kOk;
    }
    set_last_error(kErrInvalid, "dsim_batch_counts: unknown job %u", jobId);
    return kErrInvalid;
}

int dsim_batch_precision_counts(dsim_batch* b, uint32_t jobId, uint64_t out[2]) {
    if (!b || !out) return kErrInvalid;
    for (size_t k = 0; k < b->jobs.size(); k++) {
        if (b->jobs[k].id != jobId) continue;
        unsigned long long c[4];
        DSIM_CUDA_TRY(cudaMemcpyAsync(c, b->d_counts + 4 * k, 32, cudaMemcpyDeviceToHost, b->st));
        DSIM_CUDA_TRY(cudaStreamSynchronize(b->st));
        out[0] = c[2]; out[1] = c[3];
        return kOk;
    }
    set_last_error(kErrInvalid, "dsim_batch_precision_counts: unknown job %u", jobId);
    return kErrInvalid;
}

uint32_t dsim_batch_status(dsim_batch* b) {
    if (!b) return 0;
    uint32_t s = 0;
    if (cudaMemcpyAsync(&s, b->d_status, 4, cudaMemcpyDeviceToHost, b->st) != cudaSuccess ||
        cudaStreamSynchronize(b->st) != cudaSuccess)
        return 0xFFFFFFFFu;
    return s;
}

int dsim_batch_retire(dsim_batch* b, uint32_t jobId) {
    BatchJob* j = b ? find_job(b, jobId) : nullptr;
    if (!j) { set_last_error(kErrInvalid, "dsim_batch_retire: unknown job %u", jobId); return kErrInvalid; }
    j->retired = true;
    return kOk;
}

int dsim_batch_compact(dsim_batch* b) {
    if (!b) return kErrInvalid;
    bool any = false;
    for (auto& j : b->jobs) any |= j.retired;
    if (!any) return kOk;
    const size_t nj = b->jobs.size();
    std::vector<int32_t> map(nj, -1);
    std::vector<int64_t> shift(nj, 0);
    std::vector<BatchJob> kept;
    std::vector<unsigned long long> oldCounts(4 * nj), newCounts;
    if (nj) {
        DSIM_CUDA_TRY(cudaMemcpyAsync(oldCounts.data(), b->d_counts, 32 * nj, cudaMemcpyDeviceToHost, b->st));
        DSIM_CUDA_TRY(cudaStreamSynchronize(b->st));
    }
    uint64_t slot = 0;
    for (size_t k = 0; k < nj; k++) {
        BatchJob& j = b->jobs[k];
        if (j.retired) { cudaFree(j.wave); j.wave = nullptr; continue; }
        map[k] = (int32_t)kept.size();
        shift[k] = (int64_t)slot - (int64_t)j.slot0;
        slot += j.pad;
        kept.push_back(j);
        for (int q = 0; q < 4; q++) newCounts.push_back(oldCounts[4 * k + q]);
    }
    int32_t* dmap = nullptr;
    int64_t* dshift = nullptr;
    int rc;
    if ((rc = balloc(b, (void**)&dmap, nj * 4)) || (rc = balloc(b, (void**)&dshift, nj * 8))) {
        cudaFree(dmap); cudaFree(dshift);
        return rc;
    }
    b->bytes -= nj * 12;
    cudaError_t e = cudaMemcpyAsync(dmap, map.data(), nj * 4, cudaMemcpyHostToDevice, b->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dshift, shift.data(), nj * 8, cudaMemcpyHostToDevice, b->st);
    if (e == cudaSuccess && b->N) {
        k_batch_compact<<<(uint32_t)((b->N + 255) / 256), 256, 0, b->st>>>(view(b, b->cur), view(b, 1 - b->cur), dmap, dshift);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    cudaFree(dmap); cudaFree(dshift);
    if (e != cudaSuccess) { set_last_cuda_error(e, "dsim_batch_compact", __FILE__, __LINE__); return kErrCuda; }
    b->cur = 1 - b->cur;
    b->jobs = kept;
    b->N = slot;
    b->anyPrecise = b->anyLocal = b->anyPreciseCyl = b->anyLocalCyl = false;
    for (const auto& j : b->jobs) {
        const bool jc = b->subs[j.d.sub].kind == kSubCyl;
        (jc ? b->anyPreciseCyl : b->anyPrecise) |= (j.d.flags & DSIM_JOB_PRECISE) != 0;
        (jc ? b->anyLocalCyl : b->anyLocal) |= (j.d.flags & DSIM_JOB_LOCAL) != 0;
    }
    if ((rc = layout_keys(b)) || (rc = upload_jobs(b))) return rc;
    if (!newCounts.empty())
        DSIM_CUDA_TRY(cudaMemcpyAsync(b->d_counts, newCounts.data(), newCounts.size() * 8, cudaMemcpyHostToDevice, b->st));
    DSIM_CUDA_TRY(cudaStreamSynchronize(b->st));
    invalidate_graph(b);
    return kOk;
}

// Autotuner: times the same max(trialSteps, 1000) steps (a multiple of every
// candidate chunk) of the current jobs for each candidate (step-kernel
// occupancy x chunk length x fine-grid cells per reference cell edge of every
// mesh substrate) from a snapshot of the spin state, restores the snapshot and
// keeps the fastest configuration.
int dsim_batch_autotune(dsim_batch* b, uint32_t trialSteps, uint32_t best[3], float* bestMs) {
    if (!b || !best || trialSteps == 0) { set_last_error(kErrInvalid, "dsim_batch_autotune: bad argument"); return kErrInvalid; }
    if (b->N == 0) { set_last_error(kErrInvalid, "dsim_batch_autotune: no jobs"); return kErrInvalid; }
    const bool hasD = b->buf[0].d[0] != nullptr;
    const size_t words = (size_t)(kBF + kBU + (hasD ? 2 * kBD : 0)) * b->N;
    uint32_t* snap = nullptr;
    int rc = balloc(b, (void**)&snap, words * 4);
    if (rc) return rc;
    b->bytes -= words * 4;
    const size_t nj = b->jobs.size();
    std::vector<unsigned long long> counts0(4 * nj);
    auto save = [&](void) -> cudaError_t {
        cudaError_t e = cudaSuccess;
        for (int f = 0; f < kBF && e == cudaSuccess; f++)
            e = cudaMemcpyAsync(snap + (size_t)f * b->N, b->buf[b->cur].f[f], b->N * 4, cudaMemcpyDeviceToDevice, b->st);
        for (int u = 0; u < kBU && e == cudaSuccess; u++)
            e = cudaMemcpyAsync(snap + (size_t)(kBF + u) * b->N, b->buf[b->cur].u[u], b->N * 4, cudaMemcpyDeviceToDevice, b->st);
        for (int f = 0; hasD && f < kBD && e == cudaSuccess; f++)
            e = cudaMemcpyAsync(snap + (size_t)(kBF + kBU + 2 * f) * b->N, b->buf[b->cur].d[f], b->N * 8,
                                cudaMemcpyDeviceToDevice, b->st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(counts0.data(), b->d_counts, 32 * nj, cudaMemcpyDeviceToHost, b->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
        return e;
    };
    const int cur0 = b->cur;
    const uint32_t step0 = b->stepNow;
    auto restore = [&](void) -> cudaError_t {
        b->cur = cur0;
        cudaError_t e = cudaSuccess;
        for (int f = 0; f < kBF && e == cudaSuccess; f++)
            e = cudaMemcpyAsync(b->buf[b->cur].f[f], snap + (size_t)f * b->N, b->N * 4, cudaMemcpyDeviceToDevice, b->st);
        for (int u = 0; u < kBU && e == cudaSuccess; u++)
            e = cudaMemcpyAsync(b->buf[b->cur].u[u], snap + (size_t)(kBF + u) * b->N, b->N * 4, cudaMemcpyDeviceToDevice, b->st);
        for (int f = 0; hasD && f < kBD && e == cudaSuccess; f++)
            e = cudaMemcpyAsync(b->buf[b->cur].d[f], snap + (size_t)(kBF + kBU + 2 * f) * b->N, b->N * 8,
                                cudaMemcpyDeviceToDevice, b->st);
        b->stepNow = step0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_stepNow, &b->stepNow, 4, cudaMemcpyHostToDevice, b->st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_counts, counts0.data(), 32 * nj, cudaMemcpyHostToDevice, b->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
        return e;
    };
    // fine-grid resolutions: cells per reference-cell edge x 2
    const uint32_t gridHalves[] = {2, 3, 4, 5};  // 1, 1.5, 2, 2.5 fine cells per reference cell
    const uint32_t occs[] = {4, 5, 6, 8};
    const uint32_t chunks[] = {20, 40, 100, 200, 500, 1000};
    // the same steps for every candidate (a multiple of every chunk)
    const uint32_t T = std::max<uint32_t>((trialSteps + 999u) / 1000u * 1000u, 1000u);
    bool haveMesh = false;
    for (auto* m : b->meshes) haveMesh |= (m != nullptr);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float bestT = 3.4e38f;
    uint32_t bg = 0, bo = b->occupancy, bc = b->chunk;
    const uint32_t graph0 = b->graphChunks;
    cudaError_t e = save();
    auto set_grid = [&](uint32_t halves) -> int {
        for (size_t k = 0; k < b->meshes.size(); k++) {
            if (!b->meshes[k]) continue;
            SubDev& sd = b->subs[k];
            uint32_t nf = std::min<uint32_t>(1024u, (sd.g.n * halves + 1) / 2);
            int r = mesh_rebuild_accel(const_cast<dsim_mesh*>(b->meshes[k]), nf);
            if (r) return r;
            r = mesh_views(b->meshes[k], &sd.g, &sd.acc);
            if (r) return r;
            if (cudaMemcpy(b->d_subs + k, &sd, sizeof(SubDev), cudaMemcpyHostToDevice) != cudaSuccess) return kErrCuda;
        }
        return kOk;
    };
    for (uint32_t gi = 0; gi < (haveMesh ? 4u : 1u) && e == cudaSuccess && !rc; gi++) {
        if (haveMesh && (rc = set_grid(gridHalves[gi]))) break;
        for (uint32_t oc : occs) {
            for (uint32_t ch : chunks) {
                if ((e = restore()) != cudaSuccess) break;
                b->occupancy = oc; b->chunk = ch; b->graphChunks = 0;
                invalidate_graph(b);
                cudaEventRecord(e0, b->st);
                if ((rc = dsim_batch_advance(b, T))) break;
                cudaEventRecord(e1, b->st);
                if ((e = cudaEventSynchronize(e1)) != cudaSuccess) break;
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                ms *= (float)trialSteps / (float)T;  // per trialSteps steps
                if (ms < bestT) { bestT = ms; bg = haveMesh ? gridHalves[gi] : 0; bo = oc; bc = ch; }
            }
            if (rc || e != cudaSuccess) break;
        }
    }
    if (!rc && e == cudaSuccess && haveMesh) rc = set_grid(bg);
    // then the block size of the plain step kernels at that configuration
    uint32_t bt = b->blockThreads;
    const uint32_t shapes[] = {64, 128, 256};
    float bestShape = 3.4e38f;
    for (uint32_t th : shapes) {
        if (rc || e != cudaSuccess) break;
        if ((e = restore()) != cudaSuccess) break;
        b->occupancy = bo; b->chunk = bc; b->graphChunks = 0; b->blockThreads = th;
        invalidate_graph(b);
        cudaEventRecord(e0, b->st);
        if ((rc = dsim_batch_advance(b, T))) break;
        cudaEventRecord(e1, b->st);
        if ((e = cudaEventSynchronize(e1)) != cudaSuccess) break;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        ms *= (float)trialSteps / (float)T;
        if (ms < bestShape) { bestShape = ms; bt = th; }
    }
    if (bestShape < bestT) bestT = bestShape;
    b->blockThreads = bt;
    if (!rc && e == cudaSuccess) e = restore();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(snap);
    b->occupancy = bo; b->chunk = bc; b->graphChunks = graph0;
    invalidate_graph(b);
    if (rc) return rc;
    if (e != cudaSuccess) { set_last_cuda_error(e, "dsim_batch_autotune", __FILE__, __LINE__); return kErrCuda; }
    best[0] = bo; best[1] = bc; best[2] = bg;
    if (bestMs) *bestMs = bestT;
    return kOk;
}

int dsim_batch_info(dsim_batch* b, uint64_t info[6]) {
    if (!b || !info) return kErrInvalid;
    uint64_t running = 0;
    for (const auto& j : b->jobs) running += (!j.retired && !job_finished(b, j)) ? 1 : 0;
    info[0] = b->N; info[1] = b->jobs.size(); info[2] = running; info[3] = b->bytes;
    info[4] = b->launches; info[5] = b->graphLaunches;
    return kOk;
}

int dsim_batch_sync(dsim_batch* b) {
    if (!b) return kErrInvalid;
    DSIM_CUDA_TRY(cudaStreamSynchronize(b->st));
    return kOk;
}

}  // extern "C"
