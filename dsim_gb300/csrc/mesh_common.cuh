// mesh_common.cuh -- device helpers shared by the mesh step kernels (flat.cu,
// batch.cu) and the compartment search: fine-grid coordinates and Morton
// keys, the exact triangle test on a fine-grid record, membership in a
// reference-grid cell, and the reference grid scan used as the exact fallback.
#pragma once
#include "common.cuh"
#include "engine.h"

namespace dsim {

// the fine-grid coordinate of p: floor((p + 1) / Lf) clamped to [0, nf - 1]
// (floor_small / uint_small: the values of floorf and the conversion, on the
// FP32 pipe)
__device__ __forceinline__ uint32_t fine_coord(float p, float invLf, uint32_t nf) {
    float f = floor_small((p + 1.0f) * invLf);
    f = fminf(fmaxf(f, 0.0f), (float)(nf - 1));
    return uint_small(f);
}

__host__ __device__ __forceinline__ uint32_t spread3(uint32_t v) {
    // 10 bits -> every third bit
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
__host__ __device__ __forceinline__ uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    return spread3(x) | (spread3(y) << 1) | (spread3(z) << 2);
}

// ---- the step ------------------------------------------------------------
struct FastHit {
    uint32_t t;
    float x, y, z, d2;
    uint32_t type;
};
static constexpr int kMaxHits = 4;

// reference-grid membership of triangle t in cell c: binary search of the
// ascending list
__device__ __forceinline__ bool in_ref_cell(const MeshDev& g, uint32_t c, uint32_t t) {
    uint32_t lo = __ldg(g.cell_start + c), hi = __ldg(g.cell_start + c + 1);
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        uint32_t v = __ldg(g.cell_tri + mid);
        if (v == t) return true;
        if (v < t) lo = mid + 1; else hi = mid;
    }
    return false;
}

// Membership of triangle t in reference cell c from the triangle's own cell
// record (loaded once per hit): the same answer as in_ref_cell with no
// dependent loads; a triangle in more than four cells keeps the search.
__device__ __forceinline__ bool hit_in_cell(const MeshDev& g, uint4 cells, uint32_t c, uint32_t t) {
    if (cells.x == kCellMany) return in_ref_cell(g, c, t);
    return (cells.x == c) | (cells.y == c) | (cells.z == c) | (cells.w == c);
}

// The same with the rare search out of line, for a kernel whose code size
// limits it (hit resolution tests every hit slot, so an inlined search is
// copied into each unrolled slot test): the cell-local round measured 1.5 %
// faster with it, the plain round 0.6 % slower.
static __device__ __noinline__ bool in_ref_cell_search(const MeshDev& g, uint32_t c, uint32_t t) {
    return in_ref_cell(g, c, t);
}
__device__ __forceinline__ bool hit_in_cell_compact(const MeshDev& g, uint4 cells, uint32_t c, uint32_t t) {
    if (cells.x == kCellMany) return in_ref_cell_search(g, c, t);
    return (cells.x == c) | (cells.y == c) | (cells.z == c) | (cells.w == c);
}
__device__ __forceinline__ uint4 hit_cells(const MeshDev& g, uint32_t t) {
    if (!g.tri_cells) return make_uint4(kCellMany, kCellMany, kCellMany, kCellMany);
    return __ldg(g.tri_cells + t);
}

__device__ __forceinline__ uint32_t ref_coord(float p, float L, uint32_t n) {
    float f = floorf((p + 1.0f) / L);
    float hi = (float)(n - 1);
    float mn = (hi < f) ? hi : f;
    float mx = (0.0f < mn) ? mn : 0.0f;
    return (uint32_t)mx;
}

// full test of one accel record against the sub-segment (same float
// expressions as triCollDetect); returns true and fills h on a hit
// a = {n, p1.x}, b = {p1.y, p1.z, vv, t}, u4 = {u, v.x}, v4 = {v.y, v.z, uv, uu}
__device__ __forceinline__ bool test_rec_uv(float4 a, float4 b, float4 u4, float4 v4, float ox, float oy,
                                            float oz, float dx, float dy, float dz, FastHit& h) {
    float num = a.x * (a.w - ox) + a.y * (b.x - oy) + a.z * (b.y - oz);
    float den = a.x * dx + a.y * dy + a.z * dz;
    if (!(fabsf(num) <= fabsf(den)) || num == 0.0f ||
        ((__float_as_uint(num) ^ __float_as_uint(den)) & 0x80000000u))
        return false;
    float r = num / den;
    if (!((0.0f < r) & (r < 1.0f))) return false;
    uint32_t t = __float_as_uint(b.w);
    float wx = ox + r * dx - a.w;
    float wy = oy + r * dy - b.x;
    float wz = oz + r * dz - b.y;
    float wu = wx * u4.x + wy * u4.y + wz * u4.z;
    float wv = wx * u4.w + wy * v4.x + wz * v4.y;
    float uv = v4.z, uu = v4.w, vv = b.z;
    float s = (uv * wv - vv * wu) / (uv * uv - uu * vv);
    float tt = (uv * wu - uu * wv) / (uv * uv - uu * vv);
    if (!((s >= 0.0f) & (tt >= 0.0f) & (s + tt <= 1.0f))) return false;
    h.t = t;
    h.x = ox + dx * r; h.y = oy + dy * r; h.z = oz + dz * r;
    h.d2 = (ox - h.x) * (ox - h.x) + (oy - h.y) * (oy - h.y) + (oz - h.z) * (oz - h.z);
    uint32_t type = 1;
    if ((s == 0.0f) | (tt == 0.0f) | (s + tt == 1.0f)) {
        type = 2;
        if (((s == 0.0f) & (tt == 0.0f)) | ((s == 0.0f) & (tt == 1.0f)) | ((s == 1.0f) & (tt == 0.0f)))
            type = 3;
    }
    h.type = type;
    return true;
}

// the same, reading u, v, uv, uu from the triangle's records
__device__ __forceinline__ bool test_rec(const MeshDev& g, float4 a, float4 b, float ox, float oy,
                                         float oz, float dx, float dy, float dz, FastHit& h) {
    float num = a.x * (a.w - ox) + a.y * (b.x - oy) + a.z * (b.y - oz);
    float den = a.x * dx + a.y * dy + a.z * dz;
    if (!(fabsf(num) <= fabsf(den)) || num == 0.0f ||
        ((__float_as_uint(num) ^ __float_as_uint(den)) & 0x80000000u))
        return false;
    const float4* bb = reinterpret_cast<const float4*>(g.bary + __float_as_uint(b.w));
    return test_rec_uv(a, b, __ldg(bb), __ldg(bb + 1), ox, oy, oz, dx, dy, dz, h);
}

// a 64-byte record already in registers (no dependent load)
__device__ __forceinline__ bool test_full(const AccelRecFull& r, uint32_t excl, float ox, float oy, float oz,
                                          float dx, float dy, float dz, FastHit& h) {
    if (__float_as_uint(r.b.w) == excl) return false;
    return test_rec_uv(make_float4(r.a.x, r.a.y, r.a.z, r.b.x), make_float4(r.b.y, r.b.z, r.a.w, r.b.w), r.c, r.d,
                       ox, oy, oz, dx, dy, dz, h);
}

__device__ __forceinline__ AccelRecFull load_full(const AccelRecFull* p) {
    const float4* q = reinterpret_cast<const float4*>(p);
    AccelRecFull r;
    r.a = __ldg(q); r.b = __ldg(q + 1); r.c = __ldg(q + 2); r.d = __ldg(q + 3);
    return r;
}


// Conservative plane test on a fine-grid record q = {n, n.p1}: with den the
// exact denominator of triCollDetect and na = n.p1 - n.o, the exact numerator
// differs from na by at most ~2.5e-6 for points in the box (a few float
// roundings of terms of size <= 3.5), so a margin of 1e-5 keeps every record
// whose exact test can pass (0 < num/den < 1).
static constexpr float kPlaneMargin = 1e-5f;
__device__ __forceinline__ bool plane_may_cross(float4 q, float ox, float oy, float oz, float dx,
                                                float dy, float dz) {
    float den = q.x * dx + q.y * dy + q.z * dz;
    float na = q.w - (q.x * ox + q.y * oy + q.z * oz);
    return (den > 0.0f) ? ((na > -kPlaneMargin) & (na < den + kPlaneMargin))
                        : ((den < 0.0f) & (na < kPlaneMargin) & (na > den - kPlaneMargin));
}

// exact test against triangle t from its per-triangle records
__device__ __forceinline__ bool test_tri(const MeshDev& g, uint32_t t, float ox, float oy, float oz,
                                         float dx, float dy, float dz, FastHit& h) {
    const float4* pp = reinterpret_cast<const float4*>(g.plane + t);
    const float4 a = __ldg(pp), c = __ldg(pp + 1);
    return test_rec(g, a, make_float4(c.x, c.y, c.z, __uint_as_float(t)), ox, oy, oz, dx, dy, dz, h);
}

// exact test with the plane data from a 32-byte record (p1, t) and the rest
// (vv, u, v, uv, uu) from the triangle's records, loaded only past the plane
__device__ __forceinline__ bool test_split(const MeshDev& g, float4 q, float4 pt, float ox, float oy,
                                           float oz, float dx, float dy, float dz, FastHit& h) {
    float num = q.x * (pt.x - ox) + q.y * (pt.y - oy) + q.z * (pt.z - oz);
    float den = q.x * dx + q.y * dy + q.z * dz;
    if (!(fabsf(num) <= fabsf(den)) || num == 0.0f ||
        ((__float_as_uint(num) ^ __float_as_uint(den)) & 0x80000000u))
        return false;
    float r = num / den;
    if (!((0.0f < r) & (r < 1.0f))) return false;
    const uint32_t t = __float_as_uint(pt.w);
    const float vv = __ldg(&g.plane[t].vv);
    return test_rec(g, make_float4(q.x, q.y, q.z, pt.x), make_float4(pt.y, pt.z, vv, pt.w), ox, oy, oz,
                    dx, dy, dz, h);
}

// a 16-byte record k (plane in the record, triangle index beside it)
__device__ __forceinline__ bool test_narrow(const MeshDev& g, const AccelDev& acc, uint32_t k, uint32_t excl,
                                            float ox, float oy, float oz, float dx, float dy, float dz, FastHit& h) {
    const float4 q = __ldg(&acc.rec[k].q);
    if (!plane_may_cross(q, ox, oy, oz, dx, dy, dz)) return false;
    const uint32_t t = __ldg(acc.tri + k);
    if (t == excl) return false;
    return test_tri(g, t, ox, oy, oz, dx, dy, dz, h);
}

// one fine-grid entry k against a sub-segment (any record layout)
__device__ __forceinline__ bool test_entry(const MeshDev& g, const AccelDev& acc, uint32_t k,
                                           uint32_t excl, float ox, float oy, float oz, float dx,
                                           float dy, float dz, FastHit& h) {
    if (acc.wide == 2) return test_full(load_full(acc.recf + k), excl, ox, oy, oz, dx, dy, dz, h);
    if (acc.wide) {
        const float4 q = __ldg(&acc.recw[k].q);
        if (!plane_may_cross(q, ox, oy, oz, dx, dy, dz)) return false;
        const float4 pt = __ldg(&acc.recw[k].pt);
        if (__float_as_uint(pt.w) == excl) return false;
        return test_split(g, q, pt, ox, oy, oz, dx, dy, dz, h);
    }
    return test_narrow(g, acc, k, excl, ox, oy, oz, dx, dy, dz, h);
}

// cubeCollDetect over the reference grid (dSim3/src/spinKernelCpu.cpp:311-337)
static __device__ __noinline__ void ref_scan(const MeshDev& g, float ox, float oy, float oz, float px, float py,
                                             float pz, uint32_t excluded, FastHit& best, bool& found) {
    const uint32_t n = g.n;
    const float L = g.L;
    float dx = px - ox, dy = py - oy, dz = pz - oz;
    uint32_t sx = ref_coord(ox, L, n), sy = ref_coord(oy, L, n), sz = ref_coord(oz, L, n);
    uint32_t tx = ref_coord(px, L, n), ty = ref_coord(py, L, n), tz = ref_coord(pz, L, n);
    uint32_t ix = (uint32_t)((int)(tx > sx) - (int)(tx < sx));
    uint32_t iy = (uint32_t)((int)(ty > sy) - (int)(ty < sy));
    uint32_t iz = (uint32_t)((int)(tz > sz) - (int)(tz < sz));
    found = false;
    uint32_t cx = sx;
    do {
        uint32_t cy = sy;
        do {
            uint32_t cz = sz;
            do {
                uint32_t c = n * n * cz + n * cy + cx;
                uint32_t b0 = __ldg(g.cell_start + c), b1 = __ldg(g.cell_start + c + 1);
                float bd2 = 400000000.0f;
                for (uint32_t k = b0; k < b1; k++) {
                    uint32_t t = __ldg(g.cell_tri + k);
                    if (t == excluded) continue;
                    const float4* pp = reinterpret_cast<const float4*>(g.plane + t);
                    float4 ra = __ldg(pp), rc = __ldg(pp + 1);
                    float4 rb = make_float4(rc.x, rc.y, rc.z, __uint_as_float(t));
                    FastHit h;
                    if (!test_rec(g, ra, rb, ox, oy, oz, dx, dy, dz, h)) continue;
                    if (h.d2 < bd2) { bd2 = h.d2; best = h; found = true; }
                }
                cz += iz;
            } while ((cz != tz + iz) && !found);
            cy += iy;
        } while ((cy != ty + iy) && !found);
        cx += ix;
    } while ((cx != tx + ix) && !found);
}

}  // namespace dsim
