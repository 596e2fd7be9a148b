// flat_round.cuh -- one collision round of the warp-flattened mesh step, shared
// by the single-job step kernel (flat.cu) and the multi-job batch kernel
// (batch.cu).
//
// Semantics: rfdougherty/dSim dSim3/src/spinKernelCpu.cpp:198-337 (the
// collision search over the cells of the sub-segment's box, nearest hit of the
// first reference cell with a hit, last-hit triangle excluded).  The warp
// concatenates its lanes' fine-cell boxes by a prefix sum and loads 32 cell
// ranges at once, then concatenates those cells' records and tests record j,
// j + 32, ... per lane against the owner's sub-segment (segment table in shared
// memory, owner found by a shuffle binary search).  Hits are filed in the
// owner's shared-memory slots and each owner replays the reference's rule over
// its own hits (exact reference-grid scan when the slots overflowed).
#pragma once
#include "common.cuh"
#include "engine.h"
#include "mesh_common.cuh"

namespace dsim {


static constexpr int kFlatThreads = 128;
static constexpr int kFlatWarps = kFlatThreads / 32;
static constexpr int kFlatSlots = 4;      // hits kept per owner per round
static constexpr int kFlatMaxItems = 27;  // cells per segment handled by the warp (3 x 3 x 3)

struct FlatWarp {
    // sub-segment table of the current round, by owner lane
    float ox[32], oy[32], oz[32], dx[32], dy[32], dz[32];
    uint32_t excl[32];
    uint32_t box[32];  // fine-cell box origin lo0 | lo1 << 10 | lo2 << 20
    uint32_t wd[32];   // box widths w0 | w1 << 8 | w2 << 16
    // hits filed per owner
    uint32_t n[32];
    uint32_t t[kFlatSlots][32];
    uint32_t type[kFlatSlots][32];
    float d2[kFlatSlots][32];
    float x[kFlatSlots][32];
    float y[kFlatSlots][32];
    float z[kFlatSlots][32];
};

__device__ __forceinline__ void flat_file_hit(FlatWarp& H, uint32_t owner, const FastHit& h) {
    uint32_t slot = atomicAdd(&H.n[owner], 1u);
    if (slot < (uint32_t)kFlatSlots) {
        H.t[slot][owner] = h.t; H.type[slot][owner] = h.type; H.d2[slot][owner] = h.d2;
        H.x[slot][owner] = h.x; H.y[slot][owner] = h.y; H.z[slot][owner] = h.z;
    }
}

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v, uint32_t lane) {
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// index of the first lane j with incl[j] > r (incl non-decreasing over the
// lanes); valid for r < incl[31]
__device__ __forceinline__ uint32_t warp_find(uint32_t incl, uint32_t r) {
    uint32_t pos = 0;
#pragma unroll
    for (uint32_t step = 16; step > 0; step >>= 1) {
        uint32_t v = __shfl_sync(0xFFFFFFFFu, incl, pos + step - 1);
        if (v <= r) pos += step;
    }
    return pos;
}

// Queue of a warp's 32-byte records that passed the plane test, as (record,
// owner) pairs: the rest of the exact test (with its dependent loads) runs on
// 32 of them at a time with every lane busy
static constexpr uint32_t kFlatQueue = 64;  // at most 31 left over + 32 appended
struct FlatQueue {
    uint32_t e[kFlatQueue], o[kFlatQueue];
};

// one 32-byte record already in registers against a sub-segment
__device__ __forceinline__ bool test_wide_loaded(const MeshDev& g, float4 q, float4 pt, uint32_t excl,
                                                 float ox, float oy, float oz, float dx, float dy,
                                                 float dz, FastHit& h) {
    if (!plane_may_cross(q, ox, oy, oz, dx, dy, dz)) return false;
    if (__float_as_uint(pt.w) == excl) return false;
    return test_split(g, q, pt, ox, oy, oz, dx, dy, dz, h);
}

// Staging of 32-byte records in shared memory by bulk copies (the TMA engine,
// cp.async.bulk): the records of a round's cells are taken in windows of 64;
// for each window, every lane whose cell overlaps it issues one bulk copy of
// its part (each cell's records are contiguous), completing on the warp's
// mbarrier, whose expected byte count lane 0 posts first.  Two buffers: the
// next window's copies are in flight while the current one is tested.  Waits
// are bounded: past kStageSpinLimit polls the warp records kStatusStageTimeout
// and stops stepping (its spins are not written back).
static constexpr uint32_t kStageRecs = 64;
static constexpr uint32_t kStageSpinLimit = 1u << 20;
struct __align__(128) FlatStage {
    float4 rec[2][kStageRecs][2];  // [buffer][record][q, pt]
    unsigned long long bar[2];     // one mbarrier per buffer
    uint32_t parity[2];            // the phase each buffer waits for next
    uint32_t abort;                // a wait ran out
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// lane 0 of a warp, once per kernel (before any copy)
__device__ __forceinline__ void stage_init(FlatStage* P) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&P->bar[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&P->bar[1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    P->parity[0] = P->parity[1] = 0u;
    P->abort = 0u;
}

// lane 0: the window's total bytes, posted before the copies are issued
__device__ __forceinline__ void stage_expect(FlatStage* P, uint32_t buf, uint32_t bytes) {
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}\n"
                 ::"r"(smem_u32(&P->bar[buf])), "r"(bytes) : "memory");
}

// one bulk copy of n 32-byte records (16-byte aligned source and destination)
__device__ __forceinline__ void stage_copy(FlatStage* P, uint32_t buf, uint32_t at, const AccelRecWide* src,
                                           uint32_t n) {
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // the buffer's earlier generic reads first
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
            smem_u32(&P->rec[buf][at][0])),
        "l"(src), "r"(n * 32u), "r"(smem_u32(&P->bar[buf]))
        : "memory");
}

// every lane: wait for the buffer's copies (bounded); false when it timed out
__device__ __forceinline__ bool stage_wait(FlatStage* P, uint32_t buf) {
    const uint32_t bar = smem_u32(&P->bar[buf]), par = P->parity[buf];
    uint32_t done = 0;
    for (uint32_t k = 0; k < kStageSpinLimit && !done; k++) {
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(par)
            : "memory");
    }
    __syncwarp();
    return __all_sync(0xFFFFFFFFu, done != 0u);
}

// the rest of the exact test of queued record e for owner o (plane test passed)
__device__ __forceinline__ void flat_test_queued(FlatWarp& H, const MeshDev& g, const AccelDev& acc, uint32_t e,
                                                 uint32_t o) {
    const float4 q = __ldg(&acc.recw[e].q), pt = __ldg(&acc.recw[e].pt);
    FastHit h;
    if (test_split(g, q, pt, H.ox[o], H.oy[o], H.oz[o], H.dx[o], H.dy[o], H.dz[o], h)) flat_file_hit(H, o, h);
}

// appends the lanes' surviving (e, o) to the queue (qn: warp-uniform length)
// and tests full groups of 32 from its top; all lanes call it
__device__ __forceinline__ void flat_enqueue(FlatWarp& H, FlatQueue& Q, const MeshDev& g, const AccelDev& acc,
                                             uint32_t lane, bool live, uint32_t e, uint32_t o, uint32_t& qn) {
    const uint32_t b = __ballot_sync(0xFFFFFFFFu, live);
    if (live) {
        const uint32_t at = qn + __popc(b & ((1u << lane) - 1u));
        Q.e[at] = e; Q.o[at] = o;
    }
    qn += __popc(b);
    __syncwarp();
    while (qn >= 32) {
        const uint32_t at = qn - 32 + lane;
        const uint32_t eq = Q.e[at], oq = Q.o[at];
        __syncwarp();
        qn -= 32;
        flat_test_queued(H, g, acc, eq, oq);
    }
}

// One round for every lane of the warp (all 32 lanes call it).  open: the lane
// has a sub-segment (o -> p, `excluded` = last-hit triangle) to test.  On
// return, for open lanes, found / best hold the reference's collision result
// (its FP32 tests).  LAYOUT: 1 or 2 compile only the 32- or 64-byte record
// path; 0 dispatches on acc.wide at run time (every layout).  Q (32-byte
// records only): records past the plane test are queued and finished 32 at a
// time (null: finished in place)
template <int LAYOUT = 0>
__device__ __forceinline__ void flat_round_mode(FlatWarp& H, const MeshDev& g, const AccelDev& acc,
                                                uint32_t lane, bool open, float ox, float oy, float oz,
                                                float px, float py, float pz, uint32_t excluded,
                                                bool& found, FastHit& best, FlatQueue* Q = nullptr,
                                                FlatStage* P = nullptr) {
    const uint32_t FULL = 0xFFFFFFFFu;
    const float invLf = acc.invLf;
    const uint32_t nf = acc.nf;
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
    const bool solo = open && nc > (uint32_t)kFlatMaxItems;
    const uint32_t ncw = (open && !solo) ? nc : 0u;
    H.ox[lane] = ox; H.oy[lane] = oy; H.oz[lane] = oz;
    H.dx[lane] = dx; H.dy[lane] = dy; H.dz[lane] = dz;
    H.excl[lane] = excluded;
    H.box[lane] = lo0 | (lo1 << 10) | (lo2 << 20);
    H.wd[lane] = w0 | (w1 << 8) | (w2 << 16);
    H.n[lane] = 0;
    const uint32_t iincl = warp_incl_scan(ncw, lane);
    const uint32_t iexcl = iincl - ncw;
    const uint32_t itotal = __shfl_sync(FULL, iincl, 31);
    uint32_t qn = 0;  // queue length (warp-uniform)
    __syncwarp();
    // pass 1: 32 items at a time, one cell-range load per lane
    for (uint32_t ib = 0; ib < itotal; ib += 32) {
        const uint32_t m = ib + lane;
        const uint32_t ow = min(warp_find(iincl, m), 31u);
        const uint32_t ofs = __shfl_sync(FULL, iexcl, ow);
        uint32_t b0 = 0, cnt = 0;
        if (m < itotal) {
            const uint32_t q = m - ofs;
            const uint32_t wd = H.wd[ow], bx = H.box[ow];
            const uint32_t ww1 = (wd >> 8) & 0xFFu, ww2 = wd >> 16;
            const uint32_t iz = q % ww2, r = q / ww2, iy = r % ww1, ix = r / ww1;
            const uint32_t key = morton3((bx & 1023u) + ix, ((bx >> 10) & 1023u) + iy, (bx >> 20) + iz);
            b0 = __ldg(acc.start + key);
            cnt = __ldg(acc.start + key + 1) - b0;
        }
        // pass 2: the items' records, concatenated over the warp
        const uint32_t rincl = warp_incl_scan(cnt, lane);
        const uint32_t rtotal = __shfl_sync(FULL, rincl, 31);
        const uint32_t rbase = b0 - (rincl - cnt);  // record index = rbase of its item + flat index
        if (LAYOUT == 2 || (LAYOUT == 0 && acc.wide == 2)) {
            for (uint32_t rb = 0; rb < rtotal; rb += 64) {
                const uint32_t r0 = rb + lane, r1 = rb + 32 + lane;
                const uint32_t j0 = min(warp_find(rincl, r0), 31u);
                const uint32_t j1 = min(warp_find(rincl, r1), 31u);
                const uint32_t e0 = __shfl_sync(FULL, rbase, j0) + r0;
                const uint32_t e1 = __shfl_sync(FULL, rbase, j1) + r1;
                const uint32_t o0 = __shfl_sync(FULL, ow, j0);
                const uint32_t o1 = __shfl_sync(FULL, ow, j1);
                const bool v0 = r0 < rtotal, v1 = r1 < rtotal;
                AccelRecFull f0, f1;
                if (v0) f0 = load_full(acc.recf + e0);
                if (v1) f1 = load_full(acc.recf + e1);
                FastHit h;
                if (v0 && test_full(f0, H.excl[o0], H.ox[o0], H.oy[o0], H.oz[o0], H.dx[o0], H.dy[o0], H.dz[o0], h))
                    flat_file_hit(H, o0, h);
                if (v1 && test_full(f1, H.excl[o1], H.ox[o1], H.oy[o1], H.oz[o1], H.dx[o1], H.dy[o1], H.dz[o1], h))
                    flat_file_hit(H, o1, h);
            }
        } else if (LAYOUT == 1 && P) {
            // windows of kStageRecs records staged by bulk copies, the next one in
            // flight while this one is tested; lane k's cell holds the flat
            // records [rincl - cnt, rincl) at global index b0
            const uint32_t nwin = (rtotal + kStageRecs - 1) / kStageRecs;
            const uint32_t rexcl = rincl - cnt;
            auto issue = [&](uint32_t w, uint32_t buf) {
                const uint32_t lo = w * kStageRecs, hi = min(lo + kStageRecs, rtotal);
                if (lane == 0) stage_expect(P, buf, (hi - lo) * 32u);
                __syncwarp();
                const uint32_t a = max(rexcl, lo), z = min(rincl, hi);
                if (a < z) stage_copy(P, buf, a - lo, acc.recw + b0 + (a - rexcl), z - a);
            };
            if (nwin > 0 && !P->abort) issue(0, 0);
            for (uint32_t w = 0; w < nwin && !P->abort; w++) {
                const uint32_t buf = w & 1u;
                if (w + 1 < nwin) issue(w + 1, buf ^ 1u);
                if (!stage_wait(P, buf)) {
                    // a wait ran out: wait once more (bounded) for the copies in
                    // flight to this buffer and the next, then stop the warp
                    stage_wait(P, buf);
                    if (w + 1 < nwin) stage_wait(P, buf ^ 1u);
                    if (lane == 0) P->abort = 1u;
                    __syncwarp();
                    break;
                }
                if (lane == 0) P->parity[buf] ^= 1u;
                const uint32_t lo = w * kStageRecs;
                const uint32_t r0 = lo + lane, r1 = lo + 32 + lane;
                const uint32_t j0 = min(warp_find(rincl, r0), 31u);
                const uint32_t j1 = min(warp_find(rincl, r1), 31u);
                const uint32_t o0 = __shfl_sync(FULL, ow, j0);
                const uint32_t o1 = __shfl_sync(FULL, ow, j1);
                FastHit h;
                if (r0 < rtotal && test_wide_loaded(g, P->rec[buf][lane][0], P->rec[buf][lane][1], H.excl[o0],
                                                    H.ox[o0], H.oy[o0], H.oz[o0], H.dx[o0], H.dy[o0], H.dz[o0], h))
                    flat_file_hit(H, o0, h);
                if (r1 < rtotal && test_wide_loaded(g, P->rec[buf][32 + lane][0], P->rec[buf][32 + lane][1],
                                                    H.excl[o1], H.ox[o1], H.oy[o1], H.oz[o1], H.dx[o1], H.dy[o1],
                                                    H.dz[o1], h))
                    flat_file_hit(H, o1, h);
                __syncwarp();  // the buffer's reads end before its next copies
            }
        } else if (LAYOUT == 1 || (LAYOUT == 0 && acc.wide)) {
            for (uint32_t rb = 0; rb < rtotal; rb += 64) {
                const uint32_t r0 = rb + lane, r1 = rb + 32 + lane;
                const uint32_t j0 = min(warp_find(rincl, r0), 31u);
                const uint32_t j1 = min(warp_find(rincl, r1), 31u);
                const uint32_t e0 = __shfl_sync(FULL, rbase, j0) + r0;
                const uint32_t e1 = __shfl_sync(FULL, rbase, j1) + r1;
                const uint32_t o0 = __shfl_sync(FULL, ow, j0);
                const uint32_t o1 = __shfl_sync(FULL, ow, j1);
                const bool v0 = r0 < rtotal, v1 = r1 < rtotal;
                float4 q0 = make_float4(0.f, 0.f, 0.f, 0.f), t0 = q0, q1 = q0, t1 = q0;
                if (v0) { q0 = __ldg(&acc.recw[e0].q); t0 = __ldg(&acc.recw[e0].pt); }
                if (v1) { q1 = __ldg(&acc.recw[e1].q); t1 = __ldg(&acc.recw[e1].pt); }
                if (Q) {
                    const bool s0 = v0 && __float_as_uint(t0.w) != H.excl[o0] &&
                                    plane_may_cross(q0, H.ox[o0], H.oy[o0], H.oz[o0], H.dx[o0], H.dy[o0], H.dz[o0]);
                    const bool s1 = v1 && __float_as_uint(t1.w) != H.excl[o1] &&
                                    plane_may_cross(q1, H.ox[o1], H.oy[o1], H.oz[o1], H.dx[o1], H.dy[o1], H.dz[o1]);
                    flat_enqueue(H, *Q, g, acc, lane, s0, e0, o0, qn);
                    flat_enqueue(H, *Q, g, acc, lane, s1, e1, o1, qn);
                    continue;
                }
                FastHit h;
                if (v0 && test_wide_loaded(g, q0, t0, H.excl[o0], H.ox[o0], H.oy[o0], H.oz[o0],
                                           H.dx[o0], H.dy[o0], H.dz[o0], h))
                    flat_file_hit(H, o0, h);
                if (v1 && test_wide_loaded(g, q1, t1, H.excl[o1], H.ox[o1], H.oy[o1], H.oz[o1],
                                           H.dx[o1], H.dy[o1], H.dz[o1], h))
                    flat_file_hit(H, o1, h);
            }
        } else if (LAYOUT == 0) {
            for (uint32_t rb = 0; rb < rtotal; rb += 32) {
                const uint32_t r0 = rb + lane;
                const uint32_t j0 = min(warp_find(rincl, r0), 31u);
                const uint32_t e0 = __shfl_sync(FULL, rbase, j0) + r0;
                const uint32_t o0 = __shfl_sync(FULL, ow, j0);
                FastHit h;
                if (r0 < rtotal && test_narrow(g, acc, e0, H.excl[o0], H.ox[o0], H.oy[o0], H.oz[o0],
                                               H.dx[o0], H.dy[o0], H.dz[o0], h))
                    flat_file_hit(H, o0, h);
            }
        }
    }
    if (Q && lane < qn) flat_test_queued(H, g, acc, Q->e[lane], Q->o[lane]);  // the queue's remainder
    // boxes of more than kFlatMaxItems cells (long sub-segments): the owner alone
    if (solo) {
        for (uint32_t q = 0; q < nc; q++) {
            uint32_t iz = q % w2, r = q / w2, iy = r % w1, ix = r / w1;
            uint32_t key = morton3(lo0 + ix, lo1 + iy, lo2 + iz);
            uint32_t b0 = __ldg(acc.start + key), b1 = __ldg(acc.start + key + 1);
            for (uint32_t k = b0; k < b1; k++) {
                FastHit h;
                if (test_entry(g, acc, k, excluded, ox, oy, oz, dx, dy, dz, h)) flat_file_hit(H, lane, h);
            }
        }
    }
    __syncwarp();
    found = false;
    if (!open) return;
    const uint32_t n = H.n[lane];
    if (n > (uint32_t)kFlatSlots) {
        ref_scan(g, ox, oy, oz, px, py, pz, excluded, best, found);
    } else if (n > 0) {
        // the reference's traversal of its grid over the hits filed in
        // this lane's slots (a triangle filed twice from two fine cells
        // is the same hit)
        const uint32_t gn = g.n;
        const float L = g.L;
        uint32_t sx = ref_coord(ox, L, gn), sy = ref_coord(oy, L, gn), sz = ref_coord(oz, L, gn);
        uint32_t tx = ref_coord(px, L, gn), ty = ref_coord(py, L, gn), tz = ref_coord(pz, L, gn);
        uint32_t ix = (uint32_t)((int)(tx > sx) - (int)(tx < sx));
        uint32_t iy = (uint32_t)((int)(ty > sy) - (int)(ty < sy));
        uint32_t iz = (uint32_t)((int)(tz > sz) - (int)(tz < sz));
        uint32_t bq = 0;
        // each hit's reference cells, loaded together before the walk
        uint4 hc[kFlatSlots];
#pragma unroll
        for (int q = 0; q < kFlatSlots; q++)
            hc[q] = ((uint32_t)q < n) ? hit_cells(g, H.t[q][lane]) : make_uint4(kCellNone, kCellNone, kCellNone, kCellNone);
        uint32_t cx = sx;
        do {
            uint32_t cy = sy;
            do {
                uint32_t cz = sz;
                do {
                    uint32_t c = gn * gn * cz + gn * cy + cx;
#pragma unroll
                    for (uint32_t q = 0; q < (uint32_t)kFlatSlots; q++) {
                        if (q >= n) break;
                        const uint32_t t = H.t[q][lane];
                        if (!hit_in_cell(g, hc[q], c, t)) continue;
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
}

// every record layout
__device__ __forceinline__ void flat_round(FlatWarp& H, const MeshDev& g, const AccelDev& acc, uint32_t lane,
                                           bool open, float ox, float oy, float oz, float px, float py, float pz,
                                           uint32_t excluded, bool& found, FastHit& best) {
    flat_round_mode<0>(H, g, acc, lane, open, ox, oy, oz, px, py, pz, excluded, found, best);
}

// Reflection or permeation at the round's hit `best`: the permeation interval
// [umin, umax], the compartment transition table and the mirror reflection
// of dSim3/src/spinKernelCpu.cpp:238-271 and :406-422; the hit point becomes
// the next sub-segment's start and its triangle the excluded one.
__device__ __forceinline__ void apply_hit(const MeshDev& g, const FastHit& best, float u, float perm,
                                          uint32_t reflType, float& umax, float& umin, float& ox,
                                          float& oy, float& oz, float& px, float& py, float& pz,
                                          uint32_t& comp, uint32_t& fiber, uint32_t& excluded,
                                          uint32_t& nrefl, uint32_t& nperm) {
    float thr = umax - (umax - umin) * perm;
    if (u <= thr) {
        if ((reflType == 0) | (best.type > 1)) {
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
}

}  // namespace dsim
