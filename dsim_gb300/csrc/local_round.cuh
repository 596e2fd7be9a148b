// local_round.cuh -- the FP32 cell-local form of the mesh step (DSIM_JOB_LOCAL
// batch jobs): positions as FP32 offsets from a lattice origin, FP64 only to
// re-decide near-degenerate intersections.
//
// A spin's position is origin + offset, the origin a multiple of the lattice
// edge kLatticeH = 1/16 (exact in float) and the offset an FP32 vector, kept
// in [0, kLatticeH) between steps.  Every quantity of the collision test that
// depends on position is formed in the spin's local frame: the vertex p1 -
// origin is exact in float when |p1| >= |p1 - origin| (both are multiples of
// p1's ulp) and otherwise rounded at the local coordinate's finer ulp, so the
// test differs from the reference's (dSim3/src/spinKernelCpu.cpp:354-395) only
// in that positions carry about 16x finer rounding than an absolute FP32
// coordinate.  Normals, edges and the
// reflection (:406-422) are translation-invariant.
//
// An intersection whose FP32 outcome lies within the FP32 error band of a
// decision boundary -- the crossing parameter within 16 float ulps of its
// terms of 0 or 1, or a barycentric coordinate within kLocalEpsST of an edge
// -- is decided again in FP64 on the FP64 triangle table (tri_test64) from
// the exact position origin + offset; all others keep the FP32 result.  The
// grid lookups use absolute FP32 coordinates (fine-cell boxes widened by
// kAccelEps; the reference-cell order of hits).
#pragma once
#include "prec_round.cuh"

namespace dsim {

static constexpr float kLatticeH = 0.0625f;
static constexpr float kLocalEpsST = 1e-5f;
static constexpr uint32_t kLocalRefine = 0x100u;  // hit type flag: point from FP32, refine if chosen

// per-warp table of the local form: each owner's lattice origin and the queue
// of records past the plane test
// record queue: at most 31 left over + both records of 32 lanes appended
static constexpr uint32_t kLocalQueue = 96;
struct LocalWarp {
    float gx[32], gy[32], gz[32];
    uint32_t qe[kLocalQueue], qo[kLocalQueue];  // records past the plane test
    uint32_t ft[kPrecQueue], fo[kPrecQueue];  // (triangle, owner) pairs for the FP64 re-test
};

// FP32 plane {n, n.p1}, first vertex and triangle of fine-grid record k
__device__ __forceinline__ void record_load(const AccelDev& acc, uint32_t k, bool full, float4& q, float3& p1,
                                            uint32_t& t) {
    if (full) {
        const float4* p = reinterpret_cast<const float4*>(acc.recf + k);
        const float4 a = __ldg(p), b = __ldg(p + 1);  // {n, vv}, {p1, t}
        q = make_float4(a.x, a.y, a.z, a.x * b.x + a.y * b.y + a.z * b.z);
        p1 = make_float3(b.x, b.y, b.z);
        t = __float_as_uint(b.w);
    } else {
        q = __ldg(&acc.recw[k].q);
        const float4 pt = __ldg(&acc.recw[k].pt);
        p1 = make_float3(pt.x, pt.y, pt.z);
        t = __float_as_uint(pt.w);
    }
}

// the plane test of record k for owner o in o's local frame: may the plane
// meet the sub-segment?  (na: n.p1 - n.origin - n.offset; margin as
// plane_may_cross)
__device__ __forceinline__ bool local_plane(const FlatWarp& H, const LocalWarp& Lw, float4 q, uint32_t o) {
    const float den = q.x * H.dx[o] + q.y * H.dy[o] + q.z * H.dz[o];
    const float na = (q.w - (q.x * Lw.gx[o] + q.y * Lw.gy[o] + q.z * Lw.gz[o])) -
                     (q.x * H.ox[o] + q.y * H.oy[o] + q.z * H.oz[o]);
    return (den > 0.0f) ? ((na > -kPlaneMargin) & (na < den + kPlaneMargin))
                        : ((den < 0.0f) & (na < kPlaneMargin) & (na > den - kPlaneMargin)) |
                              ((den == 0.0f) & (fabsf(na) < kPlaneMargin));
}

// the FP64 re-test of triangle t for owner o from the exact position origin +
// offset; a hit point is local to o's origin
__device__ __forceinline__ bool local_fp64(const FlatWarp& H, const LocalWarp& Lw, const MeshDev& g, uint32_t t,
                                           uint32_t o, FastHit& h, PrecCount& pc) {
    pc.exact++;
    const float gx = Lw.gx[o], gy = Lw.gy[o], gz = Lw.gz[o];
    const float dx = H.dx[o], dy = H.dy[o], dz = H.dz[o];
    const double Ox = (double)gx + (double)H.ox[o], Oy = (double)gy + (double)H.oy[o], Oz = (double)gz + (double)H.oz[o];
    double r64;
    uint32_t type;
    if (!tri_test64(g.tri64, t, Ox, Oy, Oz, (double)dx, (double)dy, (double)dz, r64, type)) return false;
    double hx, hy, hz;
    const double d2 = hit_point64(Ox, Oy, Oz, (double)dx, (double)dy, (double)dz, r64, hx, hy, hz);
    h.t = t;
    h.x = (float)(hx - (double)gx); h.y = (float)(hy - (double)gy); h.z = (float)(hz - (double)gz);
    h.d2 = (float)d2;
    h.type = type;
    return true;
}

// the exact test of triangle t (unit normal q.xyz, first vertex p1) for owner
// o in o's local frame; a hit point is local to o's origin.  A case near a
// decision boundary is decided by local_fp64 here, or (defer) left to the
// caller with `deferred` set.
__device__ __forceinline__ bool local_test_core(const FlatWarp& H, const LocalWarp& Lw, const MeshDev& g, float4 q,
                                                float3 p1, uint32_t t, uint32_t o, FastHit& h, PrecCount& pc,
                                                bool defer, bool& deferred) {
    const float gx = Lw.gx[o], gy = Lw.gy[o], gz = Lw.gz[o];
    const float ox = H.ox[o], oy = H.oy[o], oz = H.oz[o], dx = H.dx[o], dy = H.dy[o], dz = H.dz[o];
    const float ax = p1.x - gx, ay = p1.y - gy, az = p1.z - gz;
    const float bx = ax - ox, by = ay - oy, bz = az - oz;
    const float num = q.x * bx + q.y * by + q.z * bz;
    const float den = q.x * dx + q.y * dy + q.z * dz;
    const float aden = fabsf(den);
    const float mag = fabsf(q.x * bx) + fabsf(q.y * by) + fabsf(q.z * bz) + fabsf(q.x * dx) + fabsf(q.y * dy) +
                      fabsf(q.z * dz);
    const float band = 16.0f * 1.1920929e-7f * mag;
    const float sn = (den > 0.0f) ? num : -num;
    if (sn < -band || sn > aden + band) return false;
    bool near = (sn <= band) || (sn >= aden - band);
    float r = 0.0f;
    if (!near) {
        r = num / den;
        const float4* bb = reinterpret_cast<const float4*>(g.bary + t);
        const float4 u4 = __ldg(bb), v4 = __ldg(bb + 1);
        const float vv = __ldg(&g.plane[t].vv);
        const float uv = v4.z, uu = v4.w;
        const float wx = ox + r * dx - ax, wy = oy + r * dy - ay, wz = oz + r * dz - az;
        const float wu = wx * u4.x + wy * u4.y + wz * u4.z;
        const float wv = wx * u4.w + wy * v4.x + wz * v4.y;
        const float s = (uv * wv - vv * wu) / (uv * uv - uu * vv);
        const float tt = (uv * wu - uu * wv) / (uv * uv - uu * vv);
        if (!((s >= -kLocalEpsST) & (tt >= -kLocalEpsST) & (s + tt <= 1.0f + kLocalEpsST))) return false;
        near = (s <= kLocalEpsST) | (tt <= kLocalEpsST) | (s + tt >= 1.0f - kLocalEpsST);
        if (!near) {
            // FP32 point for choosing the nearest hit; the chosen one gets its
            // point again in float-float arithmetic (local_refine)
            h.t = t;
            h.x = ox + dx * r; h.y = oy + dy * r; h.z = oz + dz * r;
            h.d2 = (ox - h.x) * (ox - h.x) + (oy - h.y) * (oy - h.y) + (oz - h.z) * (oz - h.z);
            h.type = 1u | kLocalRefine;
            return true;
        }
    }
    // near a decision boundary: FP64 on the exact position
    if (defer) {
        deferred = true;
        return false;
    }
    return local_fp64(H, Lw, g, t, o, h, pc);
}

// ---- float-float arithmetic (pairs hi + lo of floats, ~48-bit significand):
// Knuth's TwoSum and the fma-based TwoProduct are error-free; the rest keeps
// the pair's error near 2^-44 relative.
struct FF {
    float hi, lo;
};
__device__ __forceinline__ FF ff_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ FF ff_two_prod(float a, float b) {
    const float p = a * b;
    return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ FF ff_norm(float hi, float lo) {
    const float s = hi + lo;
    return {s, lo - (s - hi)};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
    const FF s = ff_two_sum(a.hi, b.hi);
    return ff_norm(s.hi, s.lo + (a.lo + b.lo));
}
// n . (e - o) for float vectors: e - o exactly (TwoSum), each product exactly
// (TwoProduct) up to the small term's rounding
__device__ __forceinline__ FF ff_dot_diff(float nx, float ny, float nz, float ex, float ey, float ez, float ox,
                                          float oy, float oz) {
    const FF ux = ff_two_sum(ex, -ox), uy = ff_two_sum(ey, -oy), uz = ff_two_sum(ez, -oz);
    FF px = ff_two_prod(nx, ux.hi), py = ff_two_prod(ny, uy.hi), pz = ff_two_prod(nz, uz.hi);
    px.lo += nx * ux.lo;
    py.lo += ny * uy.lo;
    pz.lo += nz * uz.lo;
    return ff_add(ff_add(px, py), pz);
}
__device__ __forceinline__ FF ff_dot(float nx, float ny, float nz, float dx, float dy, float dz) {
    return ff_add(ff_add(ff_two_prod(nx, dx), ff_two_prod(ny, dy)), ff_two_prod(nz, dz));
}
// a / b: the float quotient and one correction from the remainder
__device__ __forceinline__ FF ff_div(FF a, FF b) {
    const float q = a.hi / b.hi;
    const FF p = ff_two_prod(q, b.hi);
    const float rem = (((a.hi - p.hi) - p.lo) + a.lo) - q * b.lo;
    return ff_norm(q, rem / b.hi);
}
// o + d r rounded once to float
__device__ __forceinline__ float ff_axpy(float o, float d, FF r) {
    FF m = ff_two_prod(d, r.hi);
    m.lo = fmaf(d, r.lo, m.lo);
    const FF s = ff_two_sum(o, m.hi);
    return s.hi + (s.lo + m.lo);
}

// The chosen hit's point from the same FP32 operands in float-float
// arithmetic, rounded once to the local frame: the float nearest the exact
// crossing (but where the exact value lies within about 2^-44 of a rounding
// boundary).  In plain FP32 the point o + d r would carry an error comparable
// to the local coordinates' finer ulp, so a spin leaving a hit could start off
// a plane it lies on (an axis-aligned plane, or a coincident membrane) and
// meet that plane again at r ~ 1e-7.  Float-float keeps this on the FP32
// pipe: GB300's FP64 rate is a small fraction of its FP32 rate.  Hits decided
// in FP64 carry their point already (no kLocalRefine).
__device__ __forceinline__ void local_refine(const MeshDev& g, float gx, float gy, float gz, float ox, float oy,
                                             float oz, float dx, float dy, float dz, FastHit& h) {
    if (!(h.type & kLocalRefine)) return;
    h.type &= ~kLocalRefine;
    const float4* pp = reinterpret_cast<const float4*>(g.plane + h.t);
    const float4 a = __ldg(pp), c = __ldg(pp + 1);  // {n, p1.x}, {p1.y, p1.z, vv, info}
    const FF num = ff_dot_diff(a.x, a.y, a.z, a.w - gx, c.x - gy, c.y - gz, ox, oy, oz);
    const FF den = ff_dot(a.x, a.y, a.z, dx, dy, dz);
    const FF r = ff_div(num, den);
    h.x = ff_axpy(ox, dx, r);
    h.y = ff_axpy(oy, dy, r);
    h.z = ff_axpy(oz, dz, r);
}

// record k of the fine grid
__device__ __forceinline__ bool local_test(const FlatWarp& H, const LocalWarp& Lw, const MeshDev& g,
                                           const AccelDev& acc, uint32_t k, bool full, uint32_t o, FastHit& h,
                                           PrecCount& pc) {
    float4 q;
    float3 p1;
    uint32_t t;
    record_load(acc, k, full, q, p1, t);
    bool deferred = false;
    return local_test_core(H, Lw, g, q, p1, t, o, h, pc, false, deferred);
}

// the same, leaving a near case to the FP64 queue: returns its triangle in
// *tdef (else 0xFFFFFFFF)
__device__ __forceinline__ bool local_test_defer(const FlatWarp& H, const LocalWarp& Lw, const MeshDev& g,
                                                 const AccelDev& acc, uint32_t k, bool full, uint32_t o, FastHit& h,
                                                 PrecCount& pc, uint32_t& tdef) {
    float4 q;
    float3 p1;
    uint32_t t;
    record_load(acc, k, full, q, p1, t);
    bool deferred = false;
    const bool hit = local_test_core(H, Lw, g, q, p1, t, o, h, pc, true, deferred);
    tdef = deferred ? t : 0xFFFFFFFFu;
    return hit;
}

// triangle t from its per-triangle records
__device__ __forceinline__ bool local_test_tri(const FlatWarp& H, const LocalWarp& Lw, const MeshDev& g,
                                               uint32_t t, uint32_t o, FastHit& h, PrecCount& pc) {
    const float4* pp = reinterpret_cast<const float4*>(g.plane + t);
    const float4 a = __ldg(pp), c = __ldg(pp + 1);  // {n, p1.x}, {p1.y, p1.z, vv, info}
    bool deferred = false;
    return local_test_core(H, Lw, g, make_float4(a.x, a.y, a.z, 0.0f), make_float3(a.w, c.x, c.y), t, o, h, pc, false,
                           deferred);
}

// appends the lanes' deferred (t, o) to the FP64 queue (fn: warp-uniform
// length) and re-tests full groups of 32 in FP64; all lanes call it
// full groups of 32 from the top of the FP64 queue (rare within a round: out
// of line, so the record loop's code stays small)
__device__ __noinline__ void local_flush64(FlatWarp& H, LocalWarp& Lw, const MeshDev& g, uint32_t lane, uint32_t& fn,
                                           PrecCount& pc) {
    while (fn >= 32) {
        const uint32_t at = fn - 32 + lane;
        const uint32_t tq = Lw.ft[at], oq = Lw.fo[at];
        __syncwarp();
        fn -= 32;
        FastHit h;
        if (local_fp64(H, Lw, g, tq, oq, h, pc)) flat_file_hit(H, oq, h);
    }
}

__device__ __forceinline__ void local_enqueue64(FlatWarp& H, LocalWarp& Lw, const MeshDev& g, uint32_t lane,
                                                uint32_t t, uint32_t o, uint32_t& fn, PrecCount& pc) {
    const bool live = t != 0xFFFFFFFFu;
    const uint32_t b = __ballot_sync(0xFFFFFFFFu, live);
    if (live) {
        const uint32_t at = fn + __popc(b & ((1u << lane) - 1u));
        Lw.ft[at] = t; Lw.fo[at] = o;
    }
    fn += __popc(b);
    __syncwarp();
    if (fn >= 32) local_flush64(H, Lw, g, lane, fn, pc);
}

// appends the lanes' surviving (k, o) to the warp's queue (qn: warp-uniform
// length) and tests full groups of 32 from its top, their near cases going to
// the FP64 queue; all lanes call it
__device__ __forceinline__ void local_enqueue(FlatWarp& H, LocalWarp& Lw, const MeshDev& g, const AccelDev& acc,
                                              bool full, uint32_t lane, bool live0, uint32_t k0, uint32_t o0,
                                              bool live1, uint32_t k1, uint32_t o1, uint32_t& qn, uint32_t& fn,
                                              PrecCount& pc, bool last) {
    // both records of the lane's pair in one append (one copy of the test
    // below); `last` (warp-uniform, after the last records) also tests the
    // partial group left at the bottom of the queue
    const uint32_t b0 = __ballot_sync(0xFFFFFFFFu, live0), b1 = __ballot_sync(0xFFFFFFFFu, live1);
    const uint32_t below = (1u << lane) - 1u;
    if (live0) {
        const uint32_t at = qn + __popc(b0 & below);
        Lw.qe[at] = k0; Lw.qo[at] = o0;
    }
    if (live1) {
        const uint32_t at = qn + __popc(b0) + __popc(b1 & below);
        Lw.qe[at] = k1; Lw.qo[at] = o1;
    }
    qn += __popc(b0) + __popc(b1);
    __syncwarp();
    while (qn >= 32 || (last && qn > 0)) {
        const uint32_t cnt = min(qn, 32u);
        const bool act = lane < cnt;
        const uint32_t at = qn - cnt + (act ? lane : 0u);
        const uint32_t kq = Lw.qe[at], oq = Lw.qo[at];
        __syncwarp();
        qn -= cnt;
        FastHit h;
        uint32_t tdef = 0xFFFFFFFFu;
        if (act && local_test_defer(H, Lw, g, acc, kq, full, oq, h, pc, tdef)) flat_file_hit(H, oq, h);
        local_enqueue64(H, Lw, g, lane, act ? tdef : 0xFFFFFFFFu, oq, fn, pc);
    }
}

// The rare paths of a round, out of line so that the record loop's code stays
// small (each holds its own copy of the exact test and the FP64 re-test).
// A lane whose cell box is too large for the warp's flattened pass: its own
// records, cell by cell.
__device__ __noinline__ void local_solo(FlatWarp& H, LocalWarp& Lw, const MeshDev& g, const AccelDev& acc, bool full,
                                        uint32_t lane, uint32_t lo0, uint32_t lo1, uint32_t lo2, uint32_t w1,
                                        uint32_t w2, uint32_t nc, uint32_t excluded, PrecCount& pc) {
    for (uint32_t q = 0; q < nc; q++) {
        const uint32_t iz = q % w2, r = q / w2, iy = r % w1, ix = r / w1;
        const uint32_t key = morton3(lo0 + ix, lo1 + iy, lo2 + iz);
        const uint32_t b0 = __ldg(acc.start + key), b1 = __ldg(acc.start + key + 1);
        for (uint32_t k = b0; k < b1; k++) {
            float4 qq; float3 p1; uint32_t t;
            record_load(acc, k, full, qq, p1, t);
            pc.records++;
            if (t == excluded || !local_plane(H, Lw, qq, lane)) continue;
            FastHit h;
            if (local_test(H, Lw, g, acc, k, full, lane, h, pc)) flat_file_hit(H, lane, h);
        }
    }
}

// A lane whose hit slots overflowed: every triangle of the reference cells
// from the start cell s towards the end cell t, in order, stopping at the
// first cell with a hit (the reference's cell walk); returns found.
__device__ __noinline__ bool local_overflow(FlatWarp& H, LocalWarp& Lw, const MeshDev& g, uint32_t lane, uint32_t sx,
                                            uint32_t sy, uint32_t sz, uint32_t tx, uint32_t ty, uint32_t tz,
                                            uint32_t ix, uint32_t iy, uint32_t iz, uint32_t excluded, FastHit& best,
                                            PrecCount& pc) {
    const uint32_t gn = g.n;
    bool found = false;
    uint32_t cx = sx;
    do {
        uint32_t cy = sy;
        do {
            uint32_t cz = sz;
            do {
                const uint32_t c = gn * gn * cz + gn * cy + cx;
                const uint32_t c0 = __ldg(g.cell_start + c), c1 = __ldg(g.cell_start + c + 1);
                float bd2 = 400000000.0f;
                for (uint32_t k = c0; k < c1; k++) {
                    const uint32_t t = __ldg(g.cell_tri + k);
                    if (t == excluded) continue;
                    FastHit h;
                    if (local_test_tri(H, Lw, g, t, lane, h, pc) && h.d2 < bd2) {
                        bd2 = h.d2; best = h; found = true;
                    }
                }
                cz += iz;
            } while ((cz != tz + iz) && !found);
            cy += iy;
        } while ((cy != ty + iy) && !found);
        cx += ix;
    } while ((cx != tx + ix) && !found);
    return found;
}

// One collision round of the local form for every lane of the warp (all 32
// lanes call it).  The sub-segment o -> p is in the lane's local frame at
// origin (gx, gy, gz); on return, for open lanes, found / best hold the
// collision result with the hit point in the same frame.  LAYOUT 1 or 2
// compiles only the 32- or 64-byte record path; 0 dispatches on acc.wide.
template <int LAYOUT = 0>
__device__ __forceinline__ void local_round(FlatWarp& H, LocalWarp& Lw, const MeshDev& g, const AccelDev& acc,
                                            uint32_t lane, bool open, float gx, float gy, float gz, float ox,
                                            float oy, float oz, float px, float py, float pz, uint32_t excluded,
                                            bool& found, FastHit& best, PrecCount& pc) {
    const uint32_t FULL = 0xFFFFFFFFu;
    const bool full = LAYOUT == 0 ? acc.wide == 2 : LAYOUT == 2;  // LAYOUT 1 / 2: one record path compiled
    const float invLf = acc.invLf;
    const uint32_t nf = acc.nf;
    const float dx = px - ox, dy = py - oy, dz = pz - oz;
    // absolute FP32 end points for the grid lookups
    const float aox = gx + ox, aoy = gy + oy, aoz = gz + oz;
    const float apx = gx + px, apy = gy + py, apz = gz + pz;
    uint32_t lo0 = 0, lo1 = 0, lo2 = 0, w0 = 0, w1 = 0, w2 = 0, nc = 0;
    if (open) {
        lo0 = fine_coord(fminf(aox, apx) - kAccelEps, invLf, nf);
        lo1 = fine_coord(fminf(aoy, apy) - kAccelEps, invLf, nf);
        lo2 = fine_coord(fminf(aoz, apz) - kAccelEps, invLf, nf);
        w0 = fine_coord(fmaxf(aox, apx) + kAccelEps, invLf, nf) - lo0 + 1;
        w1 = fine_coord(fmaxf(aoy, apy) + kAccelEps, invLf, nf) - lo1 + 1;
        w2 = fine_coord(fmaxf(aoz, apz) + kAccelEps, invLf, nf) - lo2 + 1;
        nc = w0 * w1 * w2;
    }
    const bool solo = open && nc > (uint32_t)kFlatMaxItems;
    const uint32_t ncw = (open && !solo) ? nc : 0u;
    H.ox[lane] = ox; H.oy[lane] = oy; H.oz[lane] = oz;
    H.dx[lane] = dx; H.dy[lane] = dy; H.dz[lane] = dz;
    Lw.gx[lane] = gx; Lw.gy[lane] = gy; Lw.gz[lane] = gz;
    H.excl[lane] = excluded;
    H.box[lane] = lo0 | (lo1 << 10) | (lo2 << 20);
    H.wd[lane] = w0 | (w1 << 8) | (w2 << 16);
    H.n[lane] = 0;
    const uint32_t iincl = warp_incl_scan(ncw, lane);
    const uint32_t iexcl = iincl - ncw;
    const uint32_t itotal = __shfl_sync(FULL, iincl, 31);
    uint32_t qn = 0, fn = 0;  // queue lengths (warp-uniform)
    __syncwarp();
    // the warp's records pair by pair, item block after item block, and then
    // one last pass that tests the record queue's partial group: one inlined
    // copy of the exact test for the whole round
    uint32_t ib = 0, rb = 0, rtotal = 0, rincl = 0, rbase = 0, ow = 0;
    for (;;) {
        while (rb >= rtotal && ib < itotal) {  // warp-uniform
            const uint32_t m = ib + lane;
            ow = min(warp_find(iincl, m), 31u);
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
            rincl = warp_incl_scan(cnt, lane);
            rtotal = __shfl_sync(FULL, rincl, 31);
            rbase = b0 - (rincl - cnt);
            rb = 0;
            ib += 32;
        }
        const bool more = rb < rtotal;  // warp-uniform
        bool s0 = false, s1 = false;
        uint32_t e0 = 0, e1 = 0, o0 = 0, o1 = 0;
        if (more) {
            const uint32_t r0 = rb + lane, r1 = rb + 32 + lane;
            const uint32_t j0 = min(warp_find(rincl, r0), 31u);
            const uint32_t j1 = min(warp_find(rincl, r1), 31u);
            e0 = __shfl_sync(FULL, rbase, j0) + r0;
            e1 = __shfl_sync(FULL, rbase, j1) + r1;
            o0 = __shfl_sync(FULL, ow, j0);
            o1 = __shfl_sync(FULL, ow, j1);
            if (r0 < rtotal) {
                float4 q; float3 p1; uint32_t t;
                record_load(acc, e0, full, q, p1, t);
                pc.records++;
                s0 = t != H.excl[o0] && local_plane(H, Lw, q, o0);
            }
            if (r1 < rtotal) {
                float4 q; float3 p1; uint32_t t;
                record_load(acc, e1, full, q, p1, t);
                pc.records++;
                s1 = t != H.excl[o1] && local_plane(H, Lw, q, o1);
            }
            rb += 64;
        }
        local_enqueue(H, Lw, g, acc, full, lane, s0, e0, o0, s1, e1, o1, qn, fn, pc, !more);
        if (!more) break;
    }
    {
        // the FP64 queue's remainder
        FastHit h;
        if (lane < fn && local_fp64(H, Lw, g, Lw.ft[lane], Lw.fo[lane], h, pc)) flat_file_hit(H, Lw.fo[lane], h);
    }
    if (solo) local_solo(H, Lw, g, acc, full, lane, lo0, lo1, lo2, w1, w2, nc, excluded, pc);
    __syncwarp();
    found = false;
    if (!open) return;
    const uint32_t n = H.n[lane];
    const uint32_t gn = g.n;
    const float L = g.L;
    const uint32_t sx = ref_coord(aox, L, gn), sy = ref_coord(aoy, L, gn), sz = ref_coord(aoz, L, gn);
    const uint32_t tx = ref_coord(apx, L, gn), ty = ref_coord(apy, L, gn), tz = ref_coord(apz, L, gn);
    const uint32_t ix = (uint32_t)((int)(tx > sx) - (int)(tx < sx));
    const uint32_t iy = (uint32_t)((int)(ty > sy) - (int)(ty < sy));
    const uint32_t iz = (uint32_t)((int)(tz > sz) - (int)(tz < sz));
    if (n > (uint32_t)kFlatSlots) {
        found = local_overflow(H, Lw, g, lane, sx, sy, sz, tx, ty, tz, ix, iy, iz, excluded, best, pc);
        if (found) local_refine(g, gx, gy, gz, ox, oy, oz, dx, dy, dz, best);
        return;
    }
    if (n == 0) return;
    uint32_t bq = 0;
    uint4 hc[kFlatSlots];  // each hit's reference cells, loaded together before the walk
#pragma unroll
    for (int q = 0; q < kFlatSlots; q++)
        hc[q] = ((uint32_t)q < n) ? hit_cells(g, H.t[q][lane]) : make_uint4(kCellNone, kCellNone, kCellNone, kCellNone);
    uint32_t cx = sx;
    do {
        uint32_t cy = sy;
        do {
            uint32_t cz = sz;
            do {
                const uint32_t c = gn * gn * cz + gn * cy + cx;
#pragma unroll
                for (uint32_t q = 0; q < (uint32_t)kFlatSlots; q++) {
                    if (q >= n) break;
                    const uint32_t t = H.t[q][lane];
                    if (!hit_in_cell_compact(g, hc[q], c, t)) continue;
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
        local_refine(g, gx, gy, gz, ox, oy, oz, dx, dy, dz, best);
    }
}

}  // namespace dsim
