// flat.cu -- the mesh step with warp-flattened candidate lists (kernel
// variants 5-9; 8 is the default).
//
// Same semantics as the reference's collision loop
// (rfdougherty/dSim dSim3/src/spinKernelCpu.cpp:198-499): for one sub-segment
// the first cell of the reference grid (in its x-outer, z-inner traversal of
// the box between the start and end cells) whose list holds a hit gives the
// nearest hit in that list, lowest index on ties, the last-hit triangle
// excluded.  Candidates come from a finer grid whose lists hold each triangle
// in every fine cell it touches; a collision round works in two flat passes
// over the whole warp:
//
//   1. items: the lanes' fine-cell boxes are concatenated by a warp prefix sum;
//      32 items at a time, lane m finds its item's owner (binary search over
//      the prefix by shuffle) and loads that cell's record range, so 32 range
//      loads are in flight at once;
//   2. records: a second prefix sum over the 32 ranges concatenates their
//      records; lane j tests flat record j, j + 32, ... against the owner's
//      sub-segment, read from a per-warp segment table in shared memory.
//
// Hits are filed in the owner's slots and resolved by the owner: the first
// reference cell (in the reference's order) whose list holds one of its hits,
// the nearest there, the lowest index on ties; the exact reference-grid scan
// when the slots overflowed.  Lanes do not advance through the steps in
// lockstep: a lane whose step ends starts its next step in the next round, so
// one lane's chain of reflections does not idle the other 31.
#include "common.cuh"
#include "engine.h"
#include "mesh_common.cuh"

#include "flat_round.cuh"

namespace dsim {

// QUEUE (32-byte records): records past the plane test are finished 32 at a
// time from a per-warp queue (flat_round_mode's Q); STAGE: each cell's records
// staged in shared memory by bulk (TMA) copies, double-buffered
// (flat_round_mode's P)
template <bool STATS, int MINB, int LAYOUT, bool QUEUE = false, bool STAGE = false>
__global__ void __launch_bounds__(kFlatThreads, MINB) k_mesh_step_flat(MeshDev g, AccelDev acc,
                                                                       MeshStepArgs a, SpinsSorted S,
                                                                       int rng) {
    __shared__ FlatWarp wh[kFlatWarps];
    __shared__ FlatQueue wq[QUEUE ? kFlatWarps : 1];
    __shared__ FlatStage ws[STAGE ? kFlatWarps : 1];
    const uint32_t FULL = 0xFFFFFFFFu;
    const uint32_t lane = threadIdx.x & 31u;
    FlatWarp& H = wh[threadIdx.x >> 5];
    if (STAGE) {
        if (lane == 0) stage_init(&ws[threadIdx.x >> 5]);
        __syncwarp();
    }
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < S.N;
    float x = 0.0f, y = 0.0f, z = 0.0f, mag = 0.0f, phase = 0.0f;
    uint32_t comp = 0, fiber = 0, id = 0;
    if (valid) {
        x = S.x[i]; y = S.y[i]; z = S.z[i]; mag = S.mag[i]; phase = S.phase[i];
        uint32_t meta = S.meta[i];
        comp = meta & 0xFFu; fiber = meta >> 8;
        id = S.id[i];
    }
    uint32_t k0 = a.key0, k1 = a.key1;
    if (valid && rng == kRngPhiloxPerSpinKey) { k0 = a.spinKeys[2 * id]; k1 = a.spinKeys[2 * id + 1]; }
    uint32_t nrefl = 0, nperm = 0, ntested = 0, status = 0;
    // Each lane runs its own step counter: a lane whose step ends in a round
    // starts its next step in the following round, so the warp's rounds are
    // not held back by the lane with the longest reflection chain of a step.
    uint32_t it = 0;
    bool active = valid && a.iterations > 0;
    bool fresh = active;  // the lane starts step `it` at the top of the round
    Draw d;
    d.nx = d.ny = d.nz = 0.0f; d.u = 1.0f;
    float ox = x, oy = y, oz = z, px = x, py = y, pz = z;
    uint32_t excluded = 0xFFFFFFFFu, sub = 0;
    float umax = 1.0f, umin = 0.0f;
    while (__any_sync(FULL, active)) {
        if (fresh) {
            if (rng == kRngReplay) {
                float4 q = __ldg(a.draws + (size_t)it * S.N + id);
                d.nx = q.x; d.ny = q.y; d.nz = q.z; d.u = q.w;
            } else {
                d = philox_draw(a.spinBase + id, a.step0 + it, a.stream, k0, k1);
            }
            ox = x; oy = y; oz = z;
            const float sd = a.sd[comp & 3u];
            px = x + d.nx * sd; py = y + d.ny * sd; pz = z + d.nz * sd;
            // the reference's endPos equals the sub-segment target p at the top
            // of every collision round, so p doubles as endPos
            excluded = 0xFFFFFFFFu;
            umax = 1.0f; umin = 0.0f;
            sub = 0;
            if (STATS) {
                uint32_t sx = ref_coord(ox, g.L, g.n), sy = ref_coord(oy, g.L, g.n), sz = ref_coord(oz, g.L, g.n);
                uint32_t tx = ref_coord(px, g.L, g.n), ty = ref_coord(py, g.L, g.n), tz = ref_coord(pz, g.L, g.n);
                for (uint32_t cx = min(sx, tx); cx <= max(sx, tx); cx++)
                    for (uint32_t cy = min(sy, ty); cy <= max(sy, ty); cy++)
                        for (uint32_t cz = min(sz, tz); cz <= max(sz, tz); cz++) {
                            uint32_t c = g.n * g.n * cz + g.n * cy + cx;
                            ntested += __ldg(g.cell_start + c + 1) - __ldg(g.cell_start + c);
                        }
            }
            fresh = false;
        }
        const bool open = active;  // every active lane has a sub-segment to test
        {
            bool found;
            FastHit best;
            flat_round_mode<LAYOUT>(H, g, acc, lane, open, ox, oy, oz, px, py, pz, excluded, found, best,
                                    QUEUE ? &wq[threadIdx.x >> 5] : nullptr, STAGE ? &ws[threadIdx.x >> 5] : nullptr);
            if (open) {
                bool finish = !found;
                if (found) {
                    apply_hit(g, best, d.u, a.perm, a.reflType, umax, umin, ox, oy, oz, px, py, pz, comp, fiber,
                              excluded, nrefl, nperm);
                    if (++sub >= a.maxSub) {
                        status |= kStatusSubsegCap;
                        px = ox; py = oy; pz = oz;
                        finish = true;
                    }
                }
                if (finish) {
                    // end of step `it`: clamp, T2 decay, phase
                    float ex = px, ey = py, ez = pz;
                    if (ex > a.clampHi) ex = a.clampHi; else if (ex < a.clampLo) ex = a.clampLo;
                    if (ey > a.clampHi) ey = a.clampHi; else if (ey < a.clampLo) ey = a.clampLo;
                    if (ez > a.clampHi) ez = a.clampHi; else if (ez < a.clampLo) ez = a.clampLo;
                    x = ex; y = ey; z = ez;
                    mag += -mag / a.T2[comp & 3u] * a.dt;
                    float gx = a.gx, gy = a.gy, gz = a.gz;
                    if (a.grad) { float4 G = __ldg(a.grad + it); gx = G.x; gy = G.y; gz = G.z; }
                    phase += (gx * x + gy * y + gz * z) * a.pc;
                    if (++it >= a.iterations) active = false;
                    else fresh = true;
                }
            }
            __syncwarp();
            if (STAGE && ws[threadIdx.x >> 5].abort) {  // warp-uniform: a staging wait ran out
                if (valid) atomicOr(a.status, (uint32_t)kStatusStageTimeout);
                return;
            }
        }
    }
    if (!valid) return;
    S.x[i] = x; S.y[i] = y; S.z[i] = z; S.mag[i] = mag; S.phase[i] = phase;
    S.meta[i] = (comp & 0xFFu) | (fiber << 8);
    if (a.counts) { a.counts[2 * id] += nrefl; a.counts[2 * id + 1] += nperm; }
    if (STATS && a.tested) a.tested[id] += ntested;
    if (status) atomicOr(a.status, status);
}

int launch_mesh_step_flat(const MeshDev& g, const AccelDev& acc, const MeshStepArgs& a,
                          const SpinsSorted& S, int rng, cudaStream_t st, int occupancy, bool queue, bool stage) {
    if (S.N == 0 || a.iterations == 0) return kOk;
    dim3 block(kFlatThreads), grid((S.N + kFlatThreads - 1) / kFlatThreads);
    // one instantiation per record layout keeps each kernel's registers to its own path
    if (a.tested) k_mesh_step_flat<true, 4, 0><<<grid, block, 0, st>>>(g, acc, a, S, rng);
    else if (acc.wide == 2) {
        if (occupancy >= 8) k_mesh_step_flat<false, 8, 2><<<grid, block, 0, st>>>(g, acc, a, S, rng);
        else if (occupancy >= 6) k_mesh_step_flat<false, 6, 2><<<grid, block, 0, st>>>(g, acc, a, S, rng);
        else k_mesh_step_flat<false, 4, 2><<<grid, block, 0, st>>>(g, acc, a, S, rng);
    } else if (acc.wide == 1 && stage) {
        k_mesh_step_flat<false, 6, 1, false, true><<<grid, block, 0, st>>>(g, acc, a, S, rng);
    } else if (acc.wide == 1 && queue) {
        // 5 blocks per SM: 96 registers with no spills (at 6: 80 registers and
        // 124 B of spills); 3 % faster on the 1M-spin walk
        k_mesh_step_flat<false, 5, 1, true><<<grid, block, 0, st>>>(g, acc, a, S, rng);
    } else if (acc.wide == 1) {
        if (occupancy >= 8) k_mesh_step_flat<false, 8, 1><<<grid, block, 0, st>>>(g, acc, a, S, rng);
        else if (occupancy >= 6) k_mesh_step_flat<false, 6, 1><<<grid, block, 0, st>>>(g, acc, a, S, rng);
        else k_mesh_step_flat<false, 4, 1><<<grid, block, 0, st>>>(g, acc, a, S, rng);
    } else {
        if (occupancy >= 6) k_mesh_step_flat<false, 6, 0><<<grid, block, 0, st>>>(g, acc, a, S, rng);
        else k_mesh_step_flat<false, 4, 0><<<grid, block, 0, st>>>(g, acc, a, S, rng);
    }
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}

}  // namespace dsim
