// accel.cu -- the fine acceleration grid of a mesh, spin sorting by fine
// cell, and the reference-layout transposes of the dSim3 drop-in.
//
// Fine grid: every triangle is listed in every fine cell it touches (a
// separating-axis test in double against the cell widened by kAccelEps), so a
// triangle that the reference's float test reports as hit by a sub-segment is
// always in the lists of the fine cells of the sub-segment's box.  The step
// kernels (flat.cu, batch.cu) collect their hits from these lists and replay
// the reference's grid traversal over them (dSim3/src/spinKernelCpu.cpp:198-395).
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
