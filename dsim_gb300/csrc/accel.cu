// accel.cu -- the fast mesh path: a fine acceleration grid, spin sorting by
// cell, and the step kernel that uses them while keeping the reference's
// collision semantics bit for bit.
//
// Semantics (rfdougherty/dSim dSim3/src/spinKernelCpu.cpp:198-395): for one
// sub-segment the reference visits the cells of its 50^3 grid in the box
// between the start and end cells (x outer, z inner) and stops at the first
// cell whose triangle list holds a hit; the result is the nearest hit in that
// list (lowest index on ties, the last-hit triangle excluded).
//
// Here every triangle the sub-segment hits is first collected from a finer
// grid whose lists hold each triangle in every fine cell it touches (a
// separating-axis test against the cell widened by kAccelEps): a triangle
// that the float test reports as hit lies within rounding of the segment, so
// it is always found.  With no
// hit (the common case) the step is done.  Otherwise the reference's
// traversal is replayed over the found hits only: a hit counts for a
// reference cell when the triangle is in that cell's (sorted) list, found by
// binary search.  The hit tests use the same float expressions as the
// reference grid path in mesh.cu, so results are identical.
//
// Spins are reordered by the Morton code of their fine cell every few steps
// so that the threads of a warp read the same cell records (broadcast loads)
// and the records of a block's cells stay in L1.  Each spin keeps a stable id
// that keys its Philox counter, its replay draws and its counters.
#include "common.cuh"
#include "engine.h"
#include "mesh_common.cuh"

namespace dsim {

// ---- build --------------------------------------------------------------
__device__ __forceinline__ void tri_fine_range(const TriPlane& P, const TriBary& B, float invLf,
                                               uint32_t nf, uint32_t lo[3], uint32_t hi[3]) {
    float p1[3] = {P.p1x, P.p1y, P.p1z};
    float u[3] = {B.ux, B.uy, B.uz};
    float v[3] = {B.vx, B.vy, B.vz};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        float a = p1[k], b = p1[k] + v[k], c = p1[k] + u[k];
        float mn = fminf(a, fminf(b, c)) - kAccelEps;
        float mx = fmaxf(a, fmaxf(b, c)) + kAccelEps;
        lo[k] = fine_coord(mn, invLf, nf);
        hi[k] = fine_coord(mx, invLf, nf);
    }
}

// Separating-axis test of a triangle (corners relative to the box centre)
// against a box of half-extent h: the triangle's plane normal and the nine
// cross products of box axes with triangle edges.  The three box axes are
// already satisfied by the cell range (the triangle's widened bounding box).
// Evaluated in double on float inputs, with the box widened by kAccelEps, so
// every cell the float triangle touches passes.
__device__ __forceinline__ bool tri_box_overlap(const double v[3][3], const double h[3]) {
    const double e0[3] = {v[1][0] - v[0][0], v[1][1] - v[0][1], v[1][2] - v[0][2]};
    const double e1[3] = {v[2][0] - v[1][0], v[2][1] - v[1][1], v[2][2] - v[1][2]};
    const double e2[3] = {v[0][0] - v[2][0], v[0][1] - v[2][1], v[0][2] - v[2][2]};
    const double* E[3] = {e0, e1, e2};
#pragma unroll
    for (int i = 0; i < 3; i++) {      // box axis i
#pragma unroll
        for (int j = 0; j < 3; j++) {  // triangle edge j: axis = unit_i x E[j]
            double a[3] = {0.0, 0.0, 0.0};
            const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
            a[i1] = -E[j][i2];
            a[i2] = E[j][i1];
            const double p0 = a[0] * v[0][0] + a[1] * v[0][1] + a[2] * v[0][2];
            const double p1 = a[0] * v[1][0] + a[1] * v[1][1] + a[2] * v[1][2];
            const double p2 = a[0] * v[2][0] + a[1] * v[2][1] + a[2] * v[2][2];
            const double r = h[0] * fabs(a[0]) + h[1] * fabs(a[1]) + h[2] * fabs(a[2]);
            const double mn = fmin(p0, fmin(p1, p2)), mx = fmax(p0, fmax(p1, p2));
            if (mn > r || mx < -r) return false;
        }
    }
    const double n[3] = {e0[1] * e1[2] - e0[2] * e1[1], e0[2] * e1[0] - e0[0] * e1[2], e0[0] * e1[1] - e0[1] * e1[0]};
    const double d = n[0] * v[0][0] + n[1] * v[0][1] + n[2] * v[0][2];
    const double r = h[0] * fabs(n[0]) + h[1] * fabs(n[1]) + h[2] * fabs(n[2]);
    return fabs(d) <= r;
}

// box of fine cell index k on one axis, widened by kAccelEps; the outermost
// cells reach to infinity because coordinates beyond the box clamp into them
__device__ __forceinline__ void cell_span(uint32_t k, uint32_t nf, double& lo, double& hi) {
    const double Lf = 2.0 / (double)nf;
    lo = (k == 0) ? -1.0e6 : -1.0 + (double)k * Lf - (double)kAccelEps;
    hi = (k == nf - 1) ? 1.0e6 : -1.0 + (double)(k + 1) * Lf + (double)kAccelEps;
}

template <bool FILL>
__global__ void k_accel_cells(uint32_t nT, const TriPlane* __restrict__ plane,
                              const TriBary* __restrict__ bary, uint32_t nf, float invLf,
                              uint32_t* counter, const uint32_t* __restrict__ start, AccelRec* rec,
                              uint32_t* tri, AccelRecWide* recw, AccelRecFull* recf) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nT) return;
    TriPlane P = plane[t];
    TriBary B = bary[t];
    uint32_t lo[3], hi[3];
    tri_fine_range(P, B, invLf, nf, lo, hi);
    // corners as the intersection test sees the triangle: p1, p1 + v, p1 + u
    const float c0[3] = {P.p1x, P.p1y, P.p1z};
    const float c1[3] = {P.p1x + B.vx, P.p1y + B.vy, P.p1z + B.vz};
    const float c2[3] = {P.p1x + B.ux, P.p1y + B.uy, P.p1z + B.uz};
    const bool many = (hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1) > 1;
    for (uint32_t x = lo[0]; x <= hi[0]; x++)
        for (uint32_t y = lo[1]; y <= hi[1]; y++)
            for (uint32_t z = lo[2]; z <= hi[2]; z++) {
                if (many) {
                    double bl[3], bh[3], ctr[3], h[3], v[3][3];
                    cell_span(x, nf, bl[0], bh[0]);
                    cell_span(y, nf, bl[1], bh[1]);
                    cell_span(z, nf, bl[2], bh[2]);
                    for (int k = 0; k < 3; k++) {
                        ctr[k] = 0.5 * (bl[k] + bh[k]);
                        h[k] = 0.5 * (bh[k] - bl[k]);
                        v[0][k] = (double)c0[k] - ctr[k];
                        v[1][k] = (double)c1[k] - ctr[k];
                        v[2][k] = (double)c2[k] - ctr[k];
                    }
                    if (!tri_box_overlap(v, h)) continue;
                }
                uint32_t key = morton3(x, y, z);
                uint32_t slot = atomicAdd(counter + key, 1u);
                if (FILL) {
                    const float4 q = make_float4(P.nx, P.ny, P.nz, P.nx * P.p1x + P.ny * P.p1y + P.nz * P.p1z);
                    if (recf) {
                        AccelRecFull r;
                        r.a = make_float4(P.nx, P.ny, P.nz, P.vv);
                        r.b = make_float4(P.p1x, P.p1y, P.p1z, __uint_as_float(t));
                        r.c = make_float4(B.ux, B.uy, B.uz, B.vx);
                        r.d = make_float4(B.vy, B.vz, B.uv, B.uu);
                        recf[start[key] + slot] = r;
                    } else if (recw) {
                        AccelRecWide r;
                        r.q = q;
                        r.pt = make_float4(P.p1x, P.p1y, P.p1z, __uint_as_float(t));
                        recw[start[key] + slot] = r;
                    } else {
                        AccelRec r;
                        r.q = q;
                        rec[start[key] + slot] = r;
                        tri[start[key] + slot] = t;
                    }
                }
            }
}

int launch_accel_cells(bool fill, uint32_t nT, const TriPlane* plane, const TriBary* bary,
                       uint32_t nf, uint32_t* counter, const uint32_t* start, AccelRec* rec,
                       uint32_t* tri, AccelRecWide* recw, cudaStream_t st, AccelRecFull* recf) {
    if (nT == 0) return kOk;
    float invLf = (float)nf / 2.0f;
    if (fill)
        k_accel_cells<true><<<(nT + 127) / 128, 128, 0, st>>>(nT, plane, bary, nf, invLf, counter, start, rec, tri, recw, recf);
    else
        k_accel_cells<false><<<(nT + 127) / 128, 128, 0, st>>>(nT, plane, bary, nf, invLf, counter, start, rec, tri, recw, recf);
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}

// ---- spin sorting (counting sort on a coarse Morton key) -----------------
__global__ void k_sort_keys(SpinsSorted S, uint32_t nb, float invLb, uint32_t* keys, uint32_t* hist) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.N) return;
    uint32_t key = morton3(fine_coord(S.x[i], invLb, nb), fine_coord(S.y[i], invLb, nb),
                           fine_coord(S.z[i], invLb, nb));
    keys[i] = key;
    atomicAdd(hist + key, 1u);
}

__global__ void k_sort_scatter(SpinsSorted S, SpinsSorted D, const uint32_t* __restrict__ keys,
                               const uint32_t* __restrict__ start, uint32_t* cursor) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.N) return;
    uint32_t key = keys[i];
    uint32_t j = start[key] + atomicAdd(cursor + key, 1u);
    D.x[j] = S.x[i]; D.y[j] = S.y[i]; D.z[j] = S.z[i];
    D.mag[j] = S.mag[i]; D.phase[j] = S.phase[i];
    D.meta[j] = S.meta[i]; D.id[j] = S.id[i];
}

int launch_sort_spins(const SpinsSorted& S, const SpinsSorted& D, uint32_t nb, uint32_t* keys,
                      uint32_t* hist, uint32_t* start, uint32_t* scratch, cudaStream_t st) {
    if (S.N == 0) return kOk;
    uint32_t nkeys = morton3(nb - 1, nb - 1, nb - 1) + 1;
    DSIM_CUDA_TRY(cudaMemsetAsync(hist, 0, (size_t)nkeys * 4, st));
    float invLb = (float)nb / 2.0f;
    k_sort_keys<<<(S.N + 255) / 256, 256, 0, st>>>(S, nb, invLb, keys, hist);
    int rc = launch_scan_exclusive(hist, start, nkeys, scratch, st);
    if (rc) return rc;
    DSIM_CUDA_TRY(cudaMemsetAsync(hist, 0, (size_t)nkeys * 4, st));
    k_sort_scatter<<<(S.N + 255) / 256, 256, 0, st>>>(S, D, keys, start, hist);
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}

template <bool STATS>
__global__ void __launch_bounds__(128) k_mesh_step_fast(MeshDev g, AccelDev acc, MeshStepArgs a,
                                                         SpinsSorted S, int rng) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.N) return;
    float x = S.x[i], y = S.y[i], z = S.z[i], mag = S.mag[i], phase = S.phase[i];
    uint32_t meta = S.meta[i];
    uint32_t comp = meta & 0xFFu, fiber = meta >> 8;
    const uint32_t id = S.id[i];
    uint32_t nrefl = 0, nperm = 0, ntested = 0, status = 0;
    uint32_t k0 = a.key0, k1 = a.key1;
    if (rng == kRngPhiloxPerSpinKey) { k0 = a.spinKeys[2 * id]; k1 = a.spinKeys[2 * id + 1]; }
    const float invLf = acc.invLf;
    const uint32_t nf = acc.nf;
    for (uint32_t it = 0; it < a.iterations; it++) {
        Draw d;
        if (rng == kRngReplay) {
            float4 q = __ldg(a.draws + (size_t)it * S.N + id);
            d.nx = q.x; d.ny = q.y; d.nz = q.z; d.u = q.w;
        } else {
            d = philox_draw(a.spinBase + id, a.step0 + it, a.stream, k0, k1);
        }
        float ox = x, oy = y, oz = z;
        float sd = a.sd[comp & 3u];
        float px = x + d.nx * sd, py = y + d.ny * sd, pz = z + d.nz * sd;
        float ex = px, ey = py, ez = pz;
        uint32_t excluded = 0xFFFFFFFFu;
        float umax = 1.0f, umin = 0.0f;
        if (STATS) {
            // reference-grid entries in the step segment's cell box
            uint32_t sx = ref_coord(ox, g.L, g.n), sy = ref_coord(oy, g.L, g.n), sz = ref_coord(oz, g.L, g.n);
            uint32_t tx = ref_coord(px, g.L, g.n), ty = ref_coord(py, g.L, g.n), tz = ref_coord(pz, g.L, g.n);
            for (uint32_t cx = min(sx, tx); cx <= max(sx, tx); cx++)
                for (uint32_t cy = min(sy, ty); cy <= max(sy, ty); cy++)
                    for (uint32_t cz = min(sz, tz); cz <= max(sz, tz); cz++) {
                        uint32_t c = g.n * g.n * cz + g.n * cy + cx;
                        ntested += __ldg(g.cell_start + c + 1) - __ldg(g.cell_start + c);
                    }
        }
        for (uint32_t sub = 0;; sub++) {
            if (sub >= a.maxSub) { status |= kStatusSubsegCap; ex = ox; ey = oy; ez = oz; break; }
            float dx = px - ox, dy = py - oy, dz = pz - oz;
            // 1. every hit triangle, from the fine grid
            uint32_t lo0 = fine_coord(fminf(ox, px) - kAccelEps, invLf, nf);
            uint32_t lo1 = fine_coord(fminf(oy, py) - kAccelEps, invLf, nf);
            uint32_t lo2 = fine_coord(fminf(oz, pz) - kAccelEps, invLf, nf);
            uint32_t hi0 = fine_coord(fmaxf(ox, px) + kAccelEps, invLf, nf);
            uint32_t hi1 = fine_coord(fmaxf(oy, py) + kAccelEps, invLf, nf);
            uint32_t hi2 = fine_coord(fmaxf(oz, pz) + kAccelEps, invLf, nf);
            FastHit hits[kMaxHits];
            int nh = 0;
            bool overflow = false;
            for (uint32_t cx = lo0; cx <= hi0; cx++)
                for (uint32_t cy = lo1; cy <= hi1; cy++)
                    for (uint32_t cz = lo2; cz <= hi2; cz++) {
                        uint32_t key = morton3(cx, cy, cz);
                        uint32_t b0 = __ldg(acc.start + key), b1 = __ldg(acc.start + key + 1);
                        for (uint32_t k = b0; k < b1; k++) {
                            FastHit h;
                            if (!test_entry(g, acc, k, excluded, ox, oy, oz, dx, dy, dz, h)) continue;
                            bool dup = false;
                            for (int q = 0; q < nh; q++) dup |= (hits[q].t == h.t);
                            if (dup) continue;
                            if (nh < kMaxHits) hits[nh++] = h; else overflow = true;
                        }
                    }
            if (nh == 0) break;
            // 2. the reference's traversal over the hits
            FastHit best;
            bool found = false;
            if (overflow) {
                ref_scan(g, ox, oy, oz, px, py, pz, excluded, best, found);
            } else {
                const uint32_t n = g.n;
                const float L = g.L;
                uint32_t sx = ref_coord(ox, L, n), sy = ref_coord(oy, L, n), sz = ref_coord(oz, L, n);
                uint32_t tx = ref_coord(px, L, n), ty = ref_coord(py, L, n), tz = ref_coord(pz, L, n);
                uint32_t ix = (uint32_t)((int)(tx > sx) - (int)(tx < sx));
                uint32_t iy = (uint32_t)((int)(ty > sy) - (int)(ty < sy));
                uint32_t iz = (uint32_t)((int)(tz > sz) - (int)(tz < sz));
                uint32_t cx = sx;
                do {
                    uint32_t cy = sy;
                    do {
                        uint32_t cz = sz;
                        do {
                            uint32_t c = n * n * cz + n * cy + cx;
                            for (int q = 0; q < nh; q++) {
                                if (!in_ref_cell(g, c, hits[q].t)) continue;
                                if (!found || hits[q].d2 < best.d2 ||
                                    (hits[q].d2 == best.d2 && hits[q].t < best.t)) {
                                    best = hits[q];
                                    found = true;
                                }
                            }
                            cz += iz;
                        } while ((cz != tz + iz) && !found);
                        cy += iy;
                    } while ((cy != ty + iy) && !found);
                    cx += ix;
                } while ((cx != tx + ix) && !found);
            }
            if (!found) break;
            float thr = umax - (umax - umin) * a.perm;
            if (d.u <= thr) {
                if ((a.reflType == 0) | (best.type > 1)) {
                    ex = ox; ey = oy; ez = oz;
                } else {
                    const float4 nn = __ldg(reinterpret_cast<const float4*>(g.plane + best.t));
                    float nx = nn.x, ny = nn.y, nz = nn.z;
                    float sx2 = px - best.x, sy2 = py - best.y, sz2 = pz - best.z;
                    ex = (1.0f - 2.0f * nx * nx) * sx2 - 2.0f * nx * ny * sy2 - 2.0f * nx * nz * sz2 + best.x;
                    ey = -2.0f * nx * ny * sx2 + (1.0f - 2.0f * ny * ny) * sy2 - 2.0f * ny * nz * sz2 + best.y;
                    ez = -2.0f * nx * nz * sx2 - 2.0f * ny * nz * sy2 + (1.0f - 2.0f * nz * nz) * sz2 + best.z;
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
            px = ex; py = ey; pz = ez;
            excluded = best.t;
        }
        if (ex > a.clampHi) ex = a.clampHi; else if (ex < a.clampLo) ex = a.clampLo;
        if (ey > a.clampHi) ey = a.clampHi; else if (ey < a.clampLo) ey = a.clampLo;
        if (ez > a.clampHi) ez = a.clampHi; else if (ez < a.clampLo) ez = a.clampLo;
        x = ex; y = ey; z = ez;
        mag += -mag / a.T2[comp & 3u] * a.dt;
        float gx = a.gx, gy = a.gy, gz = a.gz;
        if (a.grad) { float4 G = __ldg(a.grad + it); gx = G.x; gy = G.y; gz = G.z; }
        phase += (gx * x + gy * y + gz * z) * a.pc;
    }
    S.x[i] = x; S.y[i] = y; S.z[i] = z; S.mag[i] = mag; S.phase[i] = phase;
    S.meta[i] = (comp & 0xFFu) | (fiber << 8);
    if (a.counts) { a.counts[2 * id] += nrefl; a.counts[2 * id + 1] += nperm; }
    if (STATS && a.tested) a.tested[id] += ntested;
    if (status) atomicOr(a.status, status);
}

int launch_mesh_step_fast(const MeshDev& g, const AccelDev& acc, const MeshStepArgs& a,
                          const SpinsSorted& S, int rng, cudaStream_t st) {
    if (S.N == 0 || a.iterations == 0) return kOk;
    dim3 block(128), grid((S.N + 127) / 128);
    if (a.tested) k_mesh_step_fast<true><<<grid, block, 0, st>>>(g, acc, a, S, rng);
    else k_mesh_step_fast<false><<<grid, block, 0, st>>>(g, acc, a, S, rng);
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}

}  // namespace dsim

namespace dsim {
// slot order back to spin order: D[id[i]] = S[i]
__global__ void k_unpermute(SpinsSorted S, SpinsSorted D) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.N) return;
    uint32_t j = S.id[i];
    if (j >= S.N) return;
    D.x[j] = S.x[i]; D.y[j] = S.y[i]; D.z[j] = S.z[i];
    D.mag[j] = S.mag[i]; D.phase[j] = S.phase[i]; D.meta[j] = S.meta[i]; D.id[j] = j;
}

int launch_unpermute(const SpinsSorted& S, const SpinsSorted& D, cudaStream_t st) {
    if (S.N == 0) return kOk;
    k_unpermute<<<(S.N + 255) / 256, 256, 0, st>>>(S, D);
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}
}  // namespace dsim

namespace dsim {
// the reference's AoS arrays (float3 positions, 12-byte spinData) -> SoA
// work buffers in spin order (id = index)
__global__ void k_aos_to_soa(const float* __restrict__ pos, const unsigned char* __restrict__ spin,
                             SpinsSorted D) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= D.N) return;
    D.x[i] = pos[3 * i]; D.y[i] = pos[3 * i + 1]; D.z[i] = pos[3 * i + 2];
    const unsigned char* rec = spin + 12 * (size_t)i;
    D.mag[i] = *reinterpret_cast<const float*>(rec);
    D.phase[i] = *reinterpret_cast<const float*>(rec + 4);
    D.meta[i] = (uint32_t)rec[8] | ((uint32_t)(*reinterpret_cast<const uint16_t*>(rec + 10)) << 8);
    D.id[i] = i;
}

// SoA work buffers (any slot order) -> the reference's AoS arrays by id; with
// spinKeys, each spin's key is advanced for the next call
__global__ void k_soa_to_aos(SpinsSorted S, float* pos, unsigned char* spin, uint32_t* spinKeys,
                             uint32_t iterations) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.N) return;
    uint32_t j = S.id[i];
    if (j >= S.N) return;
    pos[3 * j] = S.x[i]; pos[3 * j + 1] = S.y[i]; pos[3 * j + 2] = S.z[i];
    unsigned char* rec = spin + 12 * (size_t)j;
    *reinterpret_cast<float*>(rec) = S.mag[i];
    *reinterpret_cast<float*>(rec + 4) = S.phase[i];
    rec[8] = (unsigned char)(S.meta[i] & 0xFFu);
    *reinterpret_cast<uint16_t*>(rec + 10) = (uint16_t)(S.meta[i] >> 8);
    if (spinKeys) {
        uint32_t k0 = spinKeys[2 * j], k1 = spinKeys[2 * j + 1];
        u32x4 nk = philox4x32_10({j, iterations, 0xFFFFFFFFu, 0x5EEDu}, k0, k1);
        spinKeys[2 * j] = nk.x; spinKeys[2 * j + 1] = nk.y;
    }
}

int launch_aos_to_soa(const float* pos, const void* spin, const SpinsSorted& D, cudaStream_t st) {
    if (D.N == 0) return kOk;
    k_aos_to_soa<<<(D.N + 255) / 256, 256, 0, st>>>(pos, (const unsigned char*)spin, D);
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}

int launch_soa_to_aos(const SpinsSorted& S, float* pos, void* spin, uint32_t* spinKeys,
                      uint32_t iterations, cudaStream_t st) {
    if (S.N == 0) return kOk;
    k_soa_to_aos<<<(S.N + 255) / 256, 256, 0, st>>>(S, pos, (unsigned char*)spin, spinKeys, iterations);
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}
}  // namespace dsim
