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

// Double-buffered staging of 32-byte records in shared memory: while a warp
// tests one 64-record window, each lane's two records of the next window are
// already in flight by asynchronous copies (cp.async, 16 bytes each), so the
// load latency of a window overlaps the tests of the previous one.  A lane
// reads back only the copies it issued itself.
struct FlatStage {
    float4 rec[2][32][4];  // [buffer][lane][q0, pt0, q1, pt1]
};

__device__ __forceinline__ void stage_copy16(float4* dst, const float4* src) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void stage_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void stage_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

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
            // windows of 64 records, the next one staged while this one is tested
            uint32_t e0 = 0, e1 = 0, o0 = 0, o1 = 0;
            bool v0 = false, v1 = false;
            auto locate = [&](uint32_t rb, uint32_t& a0, uint32_t& a1, uint32_t& w0_, uint32_t& w1_, bool& u0,
                              bool& u1) {
                const uint32_t r0 = rb + lane, r1 = rb + 32 + lane;
                const uint32_t j0 = min(warp_find(rincl, r0), 31u);
                const uint32_t j1 = min(warp_find(rincl, r1), 31u);
                a0 = __shfl_sync(FULL, rbase, j0) + r0;
                a1 = __shfl_sync(FULL, rbase, j1) + r1;
                w0_ = __shfl_sync(FULL, ow, j0);
                w1_ = __shfl_sync(FULL, ow, j1);
                u0 = r0 < rtotal;
                u1 = r1 < rtotal;
            };
            auto stage = [&](uint32_t buf, uint32_t a0, uint32_t a1, bool u0, bool u1) {
                float4* d = P->rec[buf][lane];
                if (u0) {
                    stage_copy16(d, &acc.recw[a0].q);
                    stage_copy16(d + 1, &acc.recw[a0].pt);
                }
                if (u1) {
                    stage_copy16(d + 2, &acc.recw[a1].q);
                    stage_copy16(d + 3, &acc.recw[a1].pt);
                }
                stage_commit();
            };
            if (rtotal > 0) {
                locate(0, e0, e1, o0, o1, v0, v1);
                stage(0, e0, e1, v0, v1);
            }
            for (uint32_t rb = 0, buf = 0; rb < rtotal; rb += 64, buf ^= 1u) {
                uint32_t n0 = 0, n1 = 0, p0 = 0, p1 = 0;
                bool u0 = false, u1 = false;
                const bool more = rb + 64 < rtotal;  // warp-uniform
                if (more) {
                    locate(rb + 64, n0, n1, p0, p1, u0, u1);
                    stage(buf ^ 1u, n0, n1, u0, u1);
                    stage_wait<1>();
                } else {
                    stage_wait<0>();
                }
                const float4* d = P->rec[buf][lane];
                FastHit h;
                if (v0 && test_wide_loaded(g, d[0], d[1], H.excl[o0], H.ox[o0], H.oy[o0], H.oz[o0], H.dx[o0],
                                           H.dy[o0], H.dz[o0], h))
                    flat_file_hit(H, o0, h);
                if (v1 && test_wide_loaded(g, d[2], d[3], H.excl[o1], H.ox[o1], H.oy[o1], H.oz[o1], H.dx[o1],
                                           H.dy[o1], H.dz[o1], h))
                    flat_file_hit(H, o1, h);
                e0 = n0; e1 = n1; o0 = p0; o1 = p1; v0 = u0; v1 = u1;
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
