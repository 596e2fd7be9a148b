// prec_round.cuh -- the precision form of the mesh step (DSIM_JOB_PRECISE
// batch jobs): the reference's step rules evaluated in FP64.
//
// The arithmetic is that of dSim3/src/spinKernelCpu.cpp (triCollDetect
// :354-395, cubeCollDetect :311-337, collDetectRectGrid :198-301, reflectPos
// :406-422, cpuIntegrate :430-499) with every position, crossing parameter,
// barycentric and reflection in double, on per-triangle helpers evaluated in
// double from the FP32 vertices (Tri64, the formulas of
// dSim3/src/spinSystem.cpp:612-648).  Expressions keep the reference's
// evaluation order and the build contracts no multiply-add, so the walk equals
// a double-precision evaluation of the reference algorithm bit for bit.
//
// FP32 only prunes: the warp-flattened passes of flat_round.cuh gather the
// fine-grid records of each sub-segment's cell box, and a record goes to the
// FP64 test unless its FP32 plane lies clearly off the sub-segment
// (plane_near, with a margin far above the FP32 error of that test).
#pragma once
#include "flat_round.cuh"

namespace dsim {

// counters of the precision form: fine-grid records examined, FP64 triangle tests
struct PrecCount {
    uint32_t records = 0, exact = 0;
};

// FP64 sub-segment table of a warp, by owner lane (the FP32 copies in
// FlatWarp drive the cell boxes and the plane pruning), and the queue of
// records that passed the pruning: (triangle, owner) pairs tested in FP64
// 32 at a time, so the FP64 test runs with every lane busy
static constexpr uint32_t kPrecQueue = 64;  // at most 31 left over + 32 appended
struct PrecWarp {
    double ox[32], oy[32], oz[32], dx[32], dy[32], dz[32];
    uint32_t qt[kPrecQueue], qo[kPrecQueue];  // past the plane pruning
    uint32_t ft[kPrecQueue], fo[kPrecQueue];  // past the barycentric pre-test: to the FP64 test
};

// May the plane (n, w = n.p1) meet the sub-segment o -> o + d?  The FP32
// value of n.p1 - n.o differs from the FP64 numerator of the exact test by
// less than ~3e-6 for points of the box (rounding of o to float <= 6e-8 per
// axis, FP32 against FP64 unit normal <= ~3e-7 relative, a few roundings of
// terms <= 3.5), and the FP32 denominator (from the difference of the rounded
// end points) from the FP64 one by far less, so a record whose FP64 crossing
// parameter lies in (0, 1) always passes.  A
// segment parallel to the plane in FP32 passes when its start lies within
// the margin.
static constexpr float kPrecMargin = 1e-5f;
__device__ __forceinline__ bool plane_near(float nx, float ny, float nz, float w, float ox, float oy, float oz,
                                           float dx, float dy, float dz) {
    const float den = nx * dx + ny * dy + nz * dz;
    const float na = w - (nx * ox + ny * oy + nz * oz);
    return (na > fminf(den, 0.0f) - kPrecMargin) & (na < fmaxf(den, 0.0f) + kPrecMargin);
}

// triCollDetect in FP64 (dSim3/src/spinKernelCpu.cpp:354-395): on a hit,
// returns true with the crossing parameter r and the hit type (1 inside, 2
// edge, 3 vertex, by exact comparison as the reference)
__device__ __forceinline__ bool tri_test64(const Tri64* __restrict__ T, uint32_t t, double ox, double oy, double oz,
                                           double dx, double dy, double dz, double& r, uint32_t& type) {
    const double2* q = reinterpret_cast<const double2*>(T + t);
    const double2 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
    const double nx = a.x, ny = a.y, nz = b.x, p1x = b.y, p1y = c.x, p1z = c.y;
    r = (nx * (p1x - ox) + ny * (p1y - oy) + nz * (p1z - oz)) / (nx * dx + ny * dy + nz * dz);
    if (!((0.0 < r) & (r < 1.0))) return false;
    const double2 e = __ldg(q + 3), f = __ldg(q + 4), g = __ldg(q + 5), h = __ldg(q + 6), k = __ldg(q + 7);
    const double ux = e.x, uy = e.y, uz = f.x, vx = f.y, vy = g.x, vz = g.y, uv = h.x, uu = h.y, vv = k.x;
    const double wu = (ox + r * dx - p1x) * ux + (oy + r * dy - p1y) * uy + (oz + r * dz - p1z) * uz;
    const double wv = (ox + r * dx - p1x) * vx + (oy + r * dy - p1y) * vy + (oz + r * dz - p1z) * vz;
    const double s = (uv * wv - vv * wu) / (uv * uv - uu * vv);
    const double tt = (uv * wu - uu * wv) / (uv * uv - uu * vv);
    if (!((s >= 0.0) & (tt >= 0.0) & (s + tt <= 1.0))) return false;
    type = 1;
    if ((s == 0.0) | (tt == 0.0) | (s + tt == 1.0)) {
        type = 2;
        if (((s == 0.0) & (tt == 0.0)) | ((s == 0.0) & (tt == 1.0)) | ((s == 1.0) & (tt == 0.0))) type = 3;
    }
    return true;
}

// the hit point and squared distance of the reference (o + (p - o) r)
__device__ __forceinline__ double hit_point64(double ox, double oy, double oz, double dx, double dy, double dz,
                                              double r, double& hx, double& hy, double& hz) {
    hx = ox + dx * r; hy = oy + dy * r; hz = oz + dz * r;
    return (ox - hx) * (ox - hx) + (oy - hy) * (oy - hy) + (oz - hz) * (oz - hz);
}

// calcCubePos in FP64 (dSim3/src/spinSystem.cpp:691-721)
__device__ __forceinline__ uint32_t ref_coord64(double p, double L, uint32_t n) {
    const double f = floor((p + 1.0) / L);
    const double hi = (double)(n - 1);
    const double mn = (hi < f) ? hi : f;
    const double mx = (0.0 < mn) ? mn : 0.0;
    return (uint32_t)mx;
}

// The same cell from an FP32 estimate: fp is p rounded to float and invL the
// float of 1 / L.  The estimate (fp + 1) invL differs from (p + 1) / L by less
// than 1e-5 (1 + |estimate|) for |p| <= 4 (three float roundings and the
// rounding of p and 1 / L, a few 1e-7 relative each), and the FP64 quotient
// from (p + 1) / L by far less; away from an integer by more than that bound
// both have the same floor, and only near a cell boundary is the FP64
// quotient evaluated.
__device__ __forceinline__ uint32_t ref_coord64_est(double p, float fp, double L, float invL, uint32_t n) {
    const float e = (fp + 1.0f) * invL;
    const float fl = floorf(e);
    const float margin = 1e-4f * (1.0f + fabsf(e));
    if (!((e - fl > margin) & (fl + 1.0f - e > margin)) || !(fabsf(fp) <= 4.0f)) return ref_coord64(p, L, n);
    const float hi = (float)(n - 1);
    const float mn = (hi < fl) ? hi : fl;
    const float mx = (0.0f < mn) ? mn : 0.0f;
    return (uint32_t)mx;
}

// FP32 plane and triangle of fine-grid record k (32- or 64-byte layout)
__device__ __forceinline__ void record_plane(const AccelDev& acc, uint32_t k, bool full, float4& q, uint32_t& t) {
    if (full) {
        const float4* p = reinterpret_cast<const float4*>(acc.recf + k);
        const float4 a = __ldg(p), b = __ldg(p + 1);  // {n, vv}, {p1, t}
        q = make_float4(a.x, a.y, a.z, a.x * b.x + a.y * b.y + a.z * b.z);
        t = __float_as_uint(b.w);
    } else {
        q = __ldg(&acc.recw[k].q);
        t = __float_as_uint(__ldg(&acc.recw[k].pt.w));
    }
}

// a hit filed by crossing parameter (bits in the x / y slots); the owner
// recomputes the point and distance in its own registers
__device__ __forceinline__ void prec_file_hit(FlatWarp& H, uint32_t owner, uint32_t t, uint32_t type, double r) {
    const uint32_t slot = atomicAdd(&H.n[owner], 1u);
    if (slot < (uint32_t)kFlatSlots) {
        H.t[slot][owner] = t; H.type[slot][owner] = type;
        H.x[slot][owner] = __int_as_float(__double2loint(r));
        H.y[slot][owner] = __int_as_float(__double2hiint(r));
    }
}

// FP32 pruning of record k for owner o: returns the triangle to test in
// FP64, or 0xFFFFFFFF
__device__ __forceinline__ uint32_t prec_prune(const FlatWarp& H, const AccelDev& acc, uint32_t k, bool full,
                                               uint32_t o, PrecCount& pc) {
    float4 q;
    uint32_t t;
    record_plane(acc, k, full, q, t);
    pc.records++;
    if (t == H.excl[o]) return 0xFFFFFFFFu;
    if (!plane_near(q.x, q.y, q.z, q.w, H.ox[o], H.oy[o], H.oz[o], H.dx[o], H.dy[o], H.dz[o])) return 0xFFFFFFFFu;
    return t;
}

// FP64 test of triangle t against owner o's sub-segment; files a hit
__device__ __forceinline__ void prec_test(FlatWarp& H, const PrecWarp& P, const MeshDev& g, uint32_t t, uint32_t o,
                                          PrecCount& pc) {
    pc.exact++;
    double r;
    uint32_t type;
    if (tri_test64(g.tri64, t, P.ox[o], P.oy[o], P.oz[o], P.dx[o], P.dy[o], P.dz[o], r, type))
        prec_file_hit(H, o, t, type, r);
}

// FP32 barycentric pre-test: false only when the crossing of t's plane lies
// clearly outside the triangle, so the FP64 test would reject it too.  The
// FP32 crossing w = o + r d - p1 (from float positions and helpers) is within
// a few 1e-7 of the FP64 one, i.e. within 2e-4 in barycentric units for edges
// of 1e-3 or more; with the angle at p1 of about 25 degrees or more and an edge
// ratio of at most 10 the Gram system amplifies that by at most ~25, far below
// the margin of 0.05.  Other triangles (and a segment parallel to the plane
// in FP32) always go to the FP64 test.
static constexpr float kPreST = 0.05f;
__device__ __forceinline__ bool prec_pretest(const FlatWarp& H, const MeshDev& g, uint32_t t, uint32_t o) {
    const float4* pp = reinterpret_cast<const float4*>(g.plane + t);
    const float4 a = __ldg(pp), c = __ldg(pp + 1);  // {n, p1.x}, {p1.y, p1.z, vv, info}
    const float4* bb = reinterpret_cast<const float4*>(g.bary + t);
    const float4 u4 = __ldg(bb), v4 = __ldg(bb + 1);  // {u, v.x}, {v.y, v.z, uv, uu}
    const float uv = v4.z, uu = v4.w, vv = c.z;
    const float mn = fminf(uu, vv), mx = fmaxf(uu, vv);
    if (!((uv * uv <= 0.82f * uu * vv) & (mx <= 100.0f * mn) & (mn >= 1e-6f))) return true;
    const float ox = H.ox[o], oy = H.oy[o], oz = H.oz[o], dx = H.dx[o], dy = H.dy[o], dz = H.dz[o];
    const float den = a.x * dx + a.y * dy + a.z * dz;
    if (den == 0.0f) return true;
    const float r = (a.x * (a.w - ox) + a.y * (c.x - oy) + a.z * (c.y - oz)) / den;
    const float wx = ox + r * dx - a.w, wy = oy + r * dy - c.x, wz = oz + r * dz - c.y;
    const float wu = wx * u4.x + wy * u4.y + wz * u4.z;
    const float wv = wx * u4.w + wy * v4.x + wz * v4.y;
    const float D = uv * uv - uu * vv;
    const float s = (uv * wv - vv * wu) / D, tt = (uv * wu - uu * wv) / D;
    return (s >= -kPreST) & (tt >= -kPreST) & (s + tt <= 1.0f + kPreST);
}

// appends the lanes' (t, o) to the FP64 queue (fn: warp-uniform length) and
// tests full groups of 32 in FP64; all lanes call it
__device__ __forceinline__ void prec_enqueue64(FlatWarp& H, PrecWarp& P, const MeshDev& g, uint32_t lane,
                                               uint32_t t, uint32_t o, uint32_t& fn, PrecCount& pc) {
    const bool live = t != 0xFFFFFFFFu;
    const uint32_t b = __ballot_sync(0xFFFFFFFFu, live);
    if (live) {
        const uint32_t at = fn + __popc(b & ((1u << lane) - 1u));
        P.ft[at] = t; P.fo[at] = o;
    }
    fn += __popc(b);
    __syncwarp();
    while (fn >= 32) {
        const uint32_t at = fn - 32 + lane;
        const uint32_t tq = P.ft[at], oq = P.fo[at];
        __syncwarp();
        fn -= 32;
        prec_test(H, P, g, tq, oq, pc);
    }
}

// appends the lanes' surviving (t, o) to the warp's queue (qn: warp-uniform
// length) and pre-tests full groups of 32 from its top, passing the
// survivors to the FP64 queue; all lanes call it
__device__ __forceinline__ void prec_enqueue(FlatWarp& H, PrecWarp& P, const MeshDev& g, uint32_t lane,
                                             uint32_t t, uint32_t o, uint32_t& qn, uint32_t& fn, PrecCount& pc) {
    const uint32_t FULL = 0xFFFFFFFFu;
    const bool live = t != 0xFFFFFFFFu;
    const uint32_t b = __ballot_sync(FULL, live);
    if (live) {
        const uint32_t at = qn + __popc(b & ((1u << lane) - 1u));
        P.qt[at] = t; P.qo[at] = o;
    }
    qn += __popc(b);
    __syncwarp();
    while (qn >= 32) {
        const uint32_t at = qn - 32 + lane;
        const uint32_t tq = P.qt[at], oq = P.qo[at];
        __syncwarp();
        qn -= 32;
        prec_enqueue64(H, P, g, lane, prec_pretest(H, g, tq, oq) ? tq : 0xFFFFFFFFu, oq, fn, pc);
    }
}

// collDetectRectGrid's cell walk over the reference grid with cubeCollDetect
// in every cell, FP64 (used when an owner's hit slots overflowed)
static __device__ __noinline__ void ref_scan64(const MeshDev& g, double ox, double oy, double oz, double px,
                                               double py, double pz, uint32_t excluded, bool& found, uint32_t& ht,
                                               uint32_t& htype, double& hx, double& hy, double& hz, PrecCount& pc) {
    const uint32_t n = g.n;
    const double L = (double)g.L;
    const double dx = px - ox, dy = py - oy, dz = pz - oz;
    const uint32_t sx = ref_coord64(ox, L, n), sy = ref_coord64(oy, L, n), sz = ref_coord64(oz, L, n);
    const uint32_t tx = ref_coord64(px, L, n), ty = ref_coord64(py, L, n), tz = ref_coord64(pz, L, n);
    const uint32_t ix = (uint32_t)((int)(tx > sx) - (int)(tx < sx));
    const uint32_t iy = (uint32_t)((int)(ty > sy) - (int)(ty < sy));
    const uint32_t iz = (uint32_t)((int)(tz > sz) - (int)(tz < sz));
    found = false;
    uint32_t cx = sx;
    do {
        uint32_t cy = sy;
        do {
            uint32_t cz = sz;
            do {
                const uint32_t c = n * n * cz + n * cy + cx;
                const uint32_t b0 = __ldg(g.cell_start + c), b1 = __ldg(g.cell_start + c + 1);
                double bd2 = 400000000.0;
                for (uint32_t k = b0; k < b1; k++) {
                    const uint32_t t = __ldg(g.cell_tri + k);
                    if (t == excluded) continue;
                    pc.exact++;
                    double r, x, y, z;
                    uint32_t type;
                    if (!tri_test64(g.tri64, t, ox, oy, oz, dx, dy, dz, r, type)) continue;
                    const double d2 = hit_point64(ox, oy, oz, dx, dy, dz, r, x, y, z);
                    if (d2 < bd2) {
                        bd2 = d2; found = true;
                        ht = t; htype = type; hx = x; hy = y; hz = z;
                    }
                }
                cz += iz;
            } while ((cz != tz + iz) && !found);
            cy += iy;
        } while ((cy != ty + iy) && !found);
        cx += ix;
    } while ((cx != tx + ix) && !found);
}

// One FP64 collision round for every lane of the warp (all 32 lanes call
// it); the counterpart of flat_round_mode.  On return, for open lanes, found
// and the hit (triangle ht, type htype, point hx, hy, hz) hold the
// reference's collision result for the sub-segment o -> p.
__device__ __forceinline__ void prec_round(FlatWarp& H, PrecWarp& P, const MeshDev& g, const AccelDev& acc,
                                           uint32_t lane, bool open, double ox, double oy, double oz, double px,
                                           double py, double pz, uint32_t excluded, bool& found, uint32_t& ht,
                                           uint32_t& htype, double& hx, double& hy, double& hz, PrecCount& pc) {
    const uint32_t FULL = 0xFFFFFFFFu;
    const bool full = acc.wide == 2;
    const float invLf = acc.invLf;
    const uint32_t nf = acc.nf;
    const double dx = px - ox, dy = py - oy, dz = pz - oz;
    const float fox = (float)ox, foy = (float)oy, foz = (float)oz;
    const float fpx = (float)px, fpy = (float)py, fpz = (float)pz;
    uint32_t lo0 = 0, lo1 = 0, lo2 = 0, w0 = 0, w1 = 0, w2 = 0, nc = 0;
    if (open) {
        lo0 = fine_coord(fminf(fox, fpx) - kAccelEps, invLf, nf);
        lo1 = fine_coord(fminf(foy, fpy) - kAccelEps, invLf, nf);
        lo2 = fine_coord(fminf(foz, fpz) - kAccelEps, invLf, nf);
        w0 = fine_coord(fmaxf(fox, fpx) + kAccelEps, invLf, nf) - lo0 + 1;
        w1 = fine_coord(fmaxf(foy, fpy) + kAccelEps, invLf, nf) - lo1 + 1;
        w2 = fine_coord(fmaxf(foz, fpz) + kAccelEps, invLf, nf) - lo2 + 1;
        nc = w0 * w1 * w2;
    }
    const bool solo = open && nc > (uint32_t)kFlatMaxItems;
    const uint32_t ncw = (open && !solo) ? nc : 0u;
    H.ox[lane] = fox; H.oy[lane] = foy; H.oz[lane] = foz;
    H.dx[lane] = fpx - fox; H.dy[lane] = fpy - foy; H.dz[lane] = fpz - foz;
    P.ox[lane] = ox; P.oy[lane] = oy; P.oz[lane] = oz;
    P.dx[lane] = dx; P.dy[lane] = dy; P.dz[lane] = dz;
    H.excl[lane] = excluded;
    H.box[lane] = lo0 | (lo1 << 10) | (lo2 << 20);
    H.wd[lane] = w0 | (w1 << 8) | (w2 << 16);
    H.n[lane] = 0;
    const uint32_t iincl = warp_incl_scan(ncw, lane);
    const uint32_t iexcl = iincl - ncw;
    const uint32_t itotal = __shfl_sync(FULL, iincl, 31);
    uint32_t qn = 0, fn = 0;  // queue lengths (warp-uniform)
    __syncwarp();
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
        const uint32_t rincl = warp_incl_scan(cnt, lane);
        const uint32_t rtotal = __shfl_sync(FULL, rincl, 31);
        const uint32_t rbase = b0 - (rincl - cnt);
        for (uint32_t rb = 0; rb < rtotal; rb += 64) {
            const uint32_t r0 = rb + lane, r1 = rb + 32 + lane;
            const uint32_t j0 = min(warp_find(rincl, r0), 31u);
            const uint32_t j1 = min(warp_find(rincl, r1), 31u);
            const uint32_t e0 = __shfl_sync(FULL, rbase, j0) + r0;
            const uint32_t e1 = __shfl_sync(FULL, rbase, j1) + r1;
            const uint32_t o0 = __shfl_sync(FULL, ow, j0);
            const uint32_t o1 = __shfl_sync(FULL, ow, j1);
            const uint32_t t0 = (r0 < rtotal) ? prec_prune(H, acc, e0, full, o0, pc) : 0xFFFFFFFFu;
            const uint32_t t1 = (r1 < rtotal) ? prec_prune(H, acc, e1, full, o1, pc) : 0xFFFFFFFFu;
            prec_enqueue(H, P, g, lane, t0, o0, qn, fn, pc);
            prec_enqueue(H, P, g, lane, t1, o1, qn, fn, pc);
        }
    }
    // the queues' remainders (fewer than 32 each)
    {
        const uint32_t tq = P.qt[lane], oq = P.qo[lane];
        const bool pass = lane < qn && prec_pretest(H, g, tq, oq);
        prec_enqueue64(H, P, g, lane, pass ? tq : 0xFFFFFFFFu, oq, fn, pc);
        if (lane < fn) prec_test(H, P, g, P.ft[lane], P.fo[lane], pc);
    }
    if (solo) {
        for (uint32_t q = 0; q < nc; q++) {
            const uint32_t iz = q % w2, r = q / w2, iy = r % w1, ix = r / w1;
            const uint32_t key = morton3(lo0 + ix, lo1 + iy, lo2 + iz);
            const uint32_t b0 = __ldg(acc.start + key), b1 = __ldg(acc.start + key + 1);
            for (uint32_t k = b0; k < b1; k++) {
                const uint32_t t = prec_prune(H, acc, k, full, lane, pc);
                if (t != 0xFFFFFFFFu) prec_test(H, P, g, t, lane, pc);
            }
        }
    }
    __syncwarp();
    found = false;
    if (!open) return;
    const uint32_t n = H.n[lane];
    if (n > (uint32_t)kFlatSlots) {
        ref_scan64(g, ox, oy, oz, px, py, pz, excluded, found, ht, htype, hx, hy, hz, pc);
        return;
    }
    if (n == 0) return;
    // the reference's cell order over the filed hits; in a cell, the nearest
    // hit, the lowest triangle index on ties (its cell lists ascend)
    const uint32_t gn = g.n;
    const double L = (double)g.L;
    const float invL = 1.0f / g.L;
    const uint32_t sx = ref_coord64_est(ox, fox, L, invL, gn), sy = ref_coord64_est(oy, foy, L, invL, gn),
                   sz = ref_coord64_est(oz, foz, L, invL, gn);
    const uint32_t tx = ref_coord64_est(px, fpx, L, invL, gn), ty = ref_coord64_est(py, fpy, L, invL, gn),
                   tz = ref_coord64_est(pz, fpz, L, invL, gn);
    const uint32_t ix = (uint32_t)((int)(tx > sx) - (int)(tx < sx));
    const uint32_t iy = (uint32_t)((int)(ty > sy) - (int)(ty < sy));
    const uint32_t iz = (uint32_t)((int)(tz > sz) - (int)(tz < sz));
    double bd2 = 0.0;
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
                    if (!hit_in_cell(g, hc[q], c, t)) continue;
                    const double r = __hiloint2double(__float_as_int(H.y[q][lane]), __float_as_int(H.x[q][lane]));
                    double x, y, z;
                    const double d2 = hit_point64(ox, oy, oz, dx, dy, dz, r, x, y, z);
                    if (!found || d2 < bd2 || (d2 == bd2 && t < ht)) {
                        found = true; bd2 = d2;
                        ht = t; htype = H.type[q][lane]; hx = x; hy = y; hz = z;
                    }
                }
                cz += iz;
            } while ((cz != tz + iz) && !found);
            cy += iy;
        } while ((cy != ty + iy) && !found);
        cx += ix;
    } while ((cx != tx + ix) && !found);
}

// Reflection or permeation at a hit, in FP64: the permeation interval, the
// compartment transition table and reflectPos of
// dSim3/src/spinKernelCpu.cpp:238-271 and :406-422
__device__ __forceinline__ void apply_hit64(const MeshDev& g, uint32_t ht, uint32_t htype, double hx, double hy,
                                            double hz, double u, double perm, uint32_t reflType, double& umax,
                                            double& umin, double& ox, double& oy, double& oz, double& px,
                                            double& py, double& pz, uint32_t& comp, uint32_t& fiber,
                                            uint32_t& excluded, uint32_t& nrefl, uint32_t& nperm) {
    const double thr = umax - (umax - umin) * perm;
    if (u <= thr) {
        if ((reflType == 0) | (htype > 1)) {
            px = ox; py = oy; pz = oz;
        } else {
            const double2* q = reinterpret_cast<const double2*>(g.tri64 + ht);
            const double2 a = __ldg(q), b = __ldg(q + 1);
            const double nx = a.x, ny = a.y, nz = b.x;
            const double sx = px - hx, sy = py - hy, sz = pz - hz;
            px = (1 - 2 * nx * nx) * sx - 2 * nx * ny * sy - 2 * nx * nz * sz + hx;
            py = -2 * nx * ny * sx + (1 - 2 * ny * ny) * sy - 2 * ny * nz * sz + hy;
            pz = -2 * nx * nz * sx - 2 * ny * nz * sy + (1 - 2 * nz * nz) * sz + hz;
        }
        umax = thr;
        nrefl++;
    } else {
        umin = thr;
        nperm++;
        const uint32_t info = __ldg(&g.plane[ht].info);
        const uint32_t membrane = info & 3u;
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
    ox = hx; oy = hy; oz = hz;
    excluded = ht;
}

}  // namespace dsim
