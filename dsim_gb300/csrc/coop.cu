// coop.cu -- warp-cooperative mesh step (the default fast path).
//
// Same semantics as k_mesh_step_fast (accel.cu) and the reference
// (rfdougherty/dSim dSim3/src/spinKernelCpu.cpp:198-499), but the candidate
// tests are spread over the warp instead of each thread walking its own
// lists: at 1M spins in a 50 um cube a warp's 32 spins sit in ~100 different
// fine cells, so per-thread lists differ in length and most lanes idle.
//
// For one collision round every lane with an open sub-segment lists the fine
// cells of its segment's bounding box; the warp then takes these (segment,
// cell) items one at a time: the owner's segment is broadcast by shuffle and
// lane j tests record j, j + 32, ... of the cell.  A lane that finds a hit
// files it in the owner's slots in shared memory.  Each owner then replays
// the reference's first-cell-with-hit rule over its hits (or, when its slots
// overflowed, scans the reference grid itself) and reflects or permeates.
#include "common.cuh"
#include "engine.h"
#include "mesh_common.cuh"

namespace dsim {

static constexpr int kCoopThreads = 128;
static constexpr int kCoopWarps = kCoopThreads / 32;
static constexpr int kSlots = 4;      // hits kept per owner per round
static constexpr int kMaxItems = 27;  // cells per segment handled cooperatively (3 x 3 x 3)

struct WarpHits {
    uint32_t n[32];
    uint32_t t[kSlots][32];
    uint32_t type[kSlots][32];
    float d2[kSlots][32];
    float x[kSlots][32];
    float y[kSlots][32];
    float z[kSlots][32];
};

__device__ __forceinline__ void file_hit(WarpHits& H, uint32_t owner, const FastHit& h) {
    uint32_t slot = atomicAdd(&H.n[owner], 1u);
    if (slot < (uint32_t)kSlots) {
        H.t[slot][owner] = h.t; H.type[slot][owner] = h.type; H.d2[slot][owner] = h.d2;
        H.x[slot][owner] = h.x; H.y[slot][owner] = h.y; H.z[slot][owner] = h.z;
    }
}

template <bool STATS, int MINB>
__global__ void __launch_bounds__(kCoopThreads, MINB) k_mesh_step_coop(MeshDev g, AccelDev acc,
                                                                       MeshStepArgs a, SpinsSorted S,
                                                                       int rng) {
    __shared__ WarpHits wh[kCoopWarps];
    const uint32_t FULL = 0xFFFFFFFFu;
    const uint32_t lane = threadIdx.x & 31u;
    WarpHits& H = wh[threadIdx.x >> 5];
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
    const float invLf = acc.invLf;
    const uint32_t nf = acc.nf;
    for (uint32_t it = 0; it < a.iterations; it++) {
        Draw d;
        d.nx = d.ny = d.nz = 0.0f; d.u = 1.0f;
        if (valid) {
            if (rng == kRngReplay) {
                float4 q = __ldg(a.draws + (size_t)it * S.N + id);
                d.nx = q.x; d.ny = q.y; d.nz = q.z; d.u = q.w;
            } else {
                d = philox_draw(a.spinBase + id, a.step0 + it, a.stream, k0, k1);
            }
        }
        float ox = x, oy = y, oz = z;
        float sd = a.sd[comp & 3u];
        float px = x + d.nx * sd, py = y + d.ny * sd, pz = z + d.nz * sd;
        // (the reference's endPos equals the sub-segment target p at the top of
        // every collision round, so p doubles as endPos)
        uint32_t excluded = 0xFFFFFFFFu;
        float umax = 1.0f, umin = 0.0f;
        if (STATS && valid) {
            uint32_t sx = ref_coord(ox, g.L, g.n), sy = ref_coord(oy, g.L, g.n), sz = ref_coord(oz, g.L, g.n);
            uint32_t tx = ref_coord(px, g.L, g.n), ty = ref_coord(py, g.L, g.n), tz = ref_coord(pz, g.L, g.n);
            for (uint32_t cx = min(sx, tx); cx <= max(sx, tx); cx++)
                for (uint32_t cy = min(sy, ty); cy <= max(sy, ty); cy++)
                    for (uint32_t cz = min(sz, tz); cz <= max(sz, tz); cz++) {
                        uint32_t c = g.n * g.n * cz + g.n * cy + cx;
                        ntested += __ldg(g.cell_start + c + 1) - __ldg(g.cell_start + c);
                    }
        }
        bool open = valid;  // this lane still has a sub-segment to test
        uint32_t sub = 0;
        while (__any_sync(FULL, open)) {
            float dx = px - ox, dy = py - oy, dz = pz - oz;
            uint32_t lo0 = 0, lo1 = 0, lo2 = 0, w0 = 0, w1 = 0, w2 = 0, nc = 0;
            if (open) {
                lo0 = fine_coord(fminf(ox, px) - kAccelEps, invLf, nf);
                lo1 = fine_coord(fminf(oy, py) - kAccelEps, invLf, nf);
                lo2 = fine_coord(fminf(oz, pz) - kAccelEps, invLf, nf);
                w0 = fine_coord(fmaxf(ox, px) + kAccelEps, invLf, nf) - lo0 + 1;
                w1 = fine_coord(fmaxf(oy, py) + kAccelEps, invLf, nf) - lo1 + 1;
                w2 = fine_coord(fmaxf(oz, pz) + kAccelEps, invLf, nf) - lo2 + 1;
                nc = w0 * w1 * w2;
            }
            H.n[lane] = 0;
            __syncwarp();
            const bool solo = open && nc > (uint32_t)kMaxItems;
            // cooperative items: q-th cell of every lane's box
            for (uint32_t q = 0; q < (uint32_t)kMaxItems; q++) {
                const bool has = open && !solo && q < nc;
                uint32_t mask = __ballot_sync(FULL, has);
                if (!mask) break;
                uint32_t myKey = 0;
                if (has) {
                    uint32_t iz = q % w2, r = q / w2, iy = r % w1, ix = r / w1;
                    myKey = morton3(lo0 + ix, lo1 + iy, lo2 + iz);
                }
                while (mask) {
                    const uint32_t l = __ffs(mask) - 1;
                    mask &= mask - 1;
                    const uint32_t key = __shfl_sync(FULL, myKey, l);
                    const float sox = __shfl_sync(FULL, ox, l), soy = __shfl_sync(FULL, oy, l),
                                soz = __shfl_sync(FULL, oz, l);
                    const float sdx = __shfl_sync(FULL, dx, l), sdy = __shfl_sync(FULL, dy, l),
                                sdz = __shfl_sync(FULL, dz, l);
                    const uint32_t excl = __shfl_sync(FULL, excluded, l);
                    const uint32_t b0 = __ldg(acc.start + key), b1 = __ldg(acc.start + key + 1);
                    for (uint32_t k = b0 + lane; k < b1; k += 32) {
                        FastHit h;
                        if (test_entry(g, acc, k, excl, sox, soy, soz, sdx, sdy, sdz, h)) file_hit(H, l, h);
                    }
                }
            }
            // boxes of more than kMaxItems cells (long sub-segments): the owner alone
            if (solo) {
                for (uint32_t q = 0; q < nc; q++) {
                    uint32_t iz = q % w2, r = q / w2, iy = r % w1, ix = r / w1;
                    uint32_t key = morton3(lo0 + ix, lo1 + iy, lo2 + iz);
                    uint32_t b0 = __ldg(acc.start + key), b1 = __ldg(acc.start + key + 1);
                    for (uint32_t k = b0; k < b1; k++) {
                        FastHit h;
                        if (test_entry(g, acc, k, excluded, ox, oy, oz, dx, dy, dz, h)) file_hit(H, lane, h);
                    }
                }
            }
            __syncwarp();
            if (open) {
                const uint32_t n = H.n[lane];
                bool found = false;
                FastHit best;
                if (n > (uint32_t)kSlots) {
                    ref_scan(g, ox, oy, oz, px, py, pz, excluded, best, found);
                } else if (n > 0) {
                    // the reference's traversal of its grid over the hits filed in
                    // this lane's slots (read in place; a triangle filed twice from
                    // two fine cells is the same hit)
                    const uint32_t gn = g.n;
                    const float L = g.L;
                    uint32_t sx = ref_coord(ox, L, gn), sy = ref_coord(oy, L, gn), sz = ref_coord(oz, L, gn);
                    uint32_t tx = ref_coord(px, L, gn), ty = ref_coord(py, L, gn), tz = ref_coord(pz, L, gn);
                    uint32_t ix = (uint32_t)((int)(tx > sx) - (int)(tx < sx));
                    uint32_t iy = (uint32_t)((int)(ty > sy) - (int)(ty < sy));
                    uint32_t iz = (uint32_t)((int)(tz > sz) - (int)(tz < sz));
                    uint32_t bq = 0;
                    uint32_t cx = sx;
                    do {
                        uint32_t cy = sy;
                        do {
                            uint32_t cz = sz;
                            do {
                                uint32_t c = gn * gn * cz + gn * cy + cx;
                                for (uint32_t q = 0; q < n; q++) {
                                    const uint32_t t = H.t[q][lane];
                                    if (!in_ref_cell(g, c, t)) continue;
                                    const float d2 = H.d2[q][lane];
                                    if (!found || d2 < H.d2[bq][lane] || (d2 == H.d2[bq][lane] && t < H.t[bq][lane])) {
                                        bq = q;
                                        found = true;
                                    }
                                }
                                cz += iz;
                            } while ((cz != tz + iz) && !found);
                            cy += iy;
                        } while ((cy != ty + iy) && !found);
                        cx += ix;
                    } while ((cx != tx + ix) && !found);
                    if (found) {
                        best.t = H.t[bq][lane]; best.type = H.type[bq][lane]; best.d2 = H.d2[bq][lane];
                        best.x = H.x[bq][lane]; best.y = H.y[bq][lane]; best.z = H.z[bq][lane];
                    }
                }
                if (!found) {
                    open = false;
                } else {
                    float thr = umax - (umax - umin) * a.perm;
                    if (d.u <= thr) {
                        if ((a.reflType == 0) | (best.type > 1)) {
                            px = ox; py = oy; pz = oz;
                        } else {
                            const float4 nn = __ldg(reinterpret_cast<const float4*>(g.plane + best.t));
                            float nx = nn.x, ny = nn.y, nz = nn.z;
                            float sx2 = px - best.x, sy2 = py - best.y, sz2 = pz - best.z;
                            px = (1.0f - 2.0f * nx * nx) * sx2 - 2.0f * nx * ny * sy2 - 2.0f * nx * nz * sz2 + best.x;
                            py = -2.0f * nx * ny * sx2 + (1.0f - 2.0f * ny * ny) * sy2 - 2.0f * ny * nz * sz2 + best.y;
                            pz = -2.0f * nx * nz * sx2 - 2.0f * ny * nz * sy2 + (1.0f - 2.0f * nz * nz) * sz2 + best.z;
                        }
                        umax = thr;
                        nrefl++;
                    } else {
                        umin = thr;
                        nperm++;
                        uint32_t info = __ldg(&g.plane[best.t].info);
                        uint32_t membrane = info & 3u;
                        if (comp == 2) {
                            if (membrane == 0) comp = 1;
                            else { comp = 0; fiber = 0xFFFFu; }
                        } else if (comp == 1) {
                            comp = 2;
                        } else if (comp == 3) {
                            comp = 0; fiber = 0xFFFFu;
                        } else {
                            fiber = (info >> 2) & 0xFFFFu;
                            comp = (membrane == 1) ? 2u : 3u;
                        }
                    }
                    ox = best.x; oy = best.y; oz = best.z;
                    excluded = best.t;
                    if (++sub >= a.maxSub) {
                        status |= kStatusSubsegCap;
                        px = ox; py = oy; pz = oz;
                        open = false;
                    }
                }
            }
            __syncwarp();
        }
        float ex = px, ey = py, ez = pz;
        if (valid) {
            if (ex > a.clampHi) ex = a.clampHi; else if (ex < a.clampLo) ex = a.clampLo;
            if (ey > a.clampHi) ey = a.clampHi; else if (ey < a.clampLo) ey = a.clampLo;
            if (ez > a.clampHi) ez = a.clampHi; else if (ez < a.clampLo) ez = a.clampLo;
            x = ex; y = ey; z = ez;
            mag += -mag / a.T2[comp & 3u] * a.dt;
            float gx = a.gx, gy = a.gy, gz = a.gz;
            if (a.grad) { float4 G = __ldg(a.grad + it); gx = G.x; gy = G.y; gz = G.z; }
            phase += (gx * x + gy * y + gz * z) * a.pc;
        }
    }
    if (!valid) return;
    S.x[i] = x; S.y[i] = y; S.z[i] = z; S.mag[i] = mag; S.phase[i] = phase;
    S.meta[i] = (comp & 0xFFu) | (fiber << 8);
    if (a.counts) { a.counts[2 * id] += nrefl; a.counts[2 * id + 1] += nperm; }
    if (STATS && a.tested) a.tested[id] += ntested;
    if (status) atomicOr(a.status, status);
}

int launch_mesh_step_coop(const MeshDev& g, const AccelDev& acc, const MeshStepArgs& a,
                          const SpinsSorted& S, int rng, cudaStream_t st, int occupancy) {
    if (S.N == 0 || a.iterations == 0) return kOk;
    dim3 block(kCoopThreads), grid((S.N + kCoopThreads - 1) / kCoopThreads);
    if (a.tested) k_mesh_step_coop<true, 4><<<grid, block, 0, st>>>(g, acc, a, S, rng);
    else if (occupancy >= 8) k_mesh_step_coop<false, 8><<<grid, block, 0, st>>>(g, acc, a, S, rng);
    else if (occupancy >= 7) k_mesh_step_coop<false, 7><<<grid, block, 0, st>>>(g, acc, a, S, rng);
    else if (occupancy >= 6) k_mesh_step_coop<false, 6><<<grid, block, 0, st>>>(g, acc, a, S, rng);
    else k_mesh_step_coop<false, 4><<<grid, block, 0, st>>>(g, acc, a, S, rng);
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}

}  // namespace dsim
