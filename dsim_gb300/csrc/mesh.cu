// mesh.cu -- triangle-mesh substrate on the GPU: exact grid build, per-triangle
// records (the step kernels are in flat.cu and batch.cu).
//
// Reference (rfdougherty/dSim):
//   cell of a point  dSim3/src/spinSystem.cpp:691-759 (calcCubePos/Hash)
//   grid membership  dSim3/src/spinSystem.cpp:1094-1379 (populateCubes,
//                    pointInCube, rayTriangleIntersect)
//   triangle helpers dSim3/src/spinSystem.cpp:612-648
// Compiled with -fmad=false: every float expression keeps the reference's
// evaluation order and rounding, so the grid and records equal the reference's.
#include "common.cuh"
#include "engine.h"

namespace dsim {

// ------------------------------------------------------------------------
// cell coordinate: std::max(0, std::min(floor((p+1)/L), n-1)) cast to uint
// ------------------------------------------------------------------------
__device__ __forceinline__ uint32_t cube_coord(float p, float L, uint32_t n) {
    float f = floorf((p + 1.0f) / L);
    float hi = (float)(n - 1);
    float mn = (hi < f) ? hi : f;
    float mx = (0.0f < mn) ? mn : 0.0f;
    return (uint32_t)mx;
}

// ------------------------------------------------------------------------
// Triangle helpers and records
// ------------------------------------------------------------------------
__device__ __forceinline__ void make_records(float x1, float y1, float z1, float x2, float y2,
                                             float z2, float x3, float y3, float z3,
                                             uint32_t info, TriPlane& P, TriBary& B) {
    float nx = (y2 - y1) * (z3 - z1) - (z2 - z1) * (y3 - y1);
    float ny = (z2 - z1) * (x3 - x1) - (x2 - x1) * (z3 - z1);
    float nz = (x2 - x1) * (y3 - y1) - (y2 - y1) * (x3 - x1);
    float length = sqrtf(nx * nx + ny * ny + nz * nz);
    P.nx = nx / length; P.ny = ny / length; P.nz = nz / length;
    P.p1x = x1; P.p1y = y1; P.p1z = z1;
    P.vv = (x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1) + (z2 - z1) * (z2 - z1);
    P.info = info;
    B.ux = x3 - x1; B.uy = y3 - y1; B.uz = z3 - z1;
    B.vx = x2 - x1; B.vy = y2 - y1; B.vz = z2 - z1;
    B.uv = (x3 - x1) * (x2 - x1) + (y3 - y1) * (y2 - y1) + (z3 - z1) * (z2 - z1);
    B.uu = (x3 - x1) * (x3 - x1) + (y3 - y1) * (y3 - y1) + (z3 - z1) * (z3 - z1);
}

// records from vertices + triangle vertex indices (native path)
__global__ void k_records_from_mesh(uint32_t nT, const float* __restrict__ V,
                                    const uint32_t* __restrict__ trgls,
                                    const uint32_t* __restrict__ membrane,
                                    const uint32_t* __restrict__ fiber, TriPlane* plane,
                                    TriBary* bary) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nT) return;
    uint32_t a = trgls[3 * t], b = trgls[3 * t + 1], c = trgls[3 * t + 2];
    TriPlane P; TriBary B;
    make_records(V[3 * a], V[3 * a + 1], V[3 * a + 2], V[3 * b], V[3 * b + 1], V[3 * b + 2],
                 V[3 * c], V[3 * c + 1], V[3 * c + 2], pack_info(membrane[t], fiber[t]), P, B);
    plane[t] = P;
    bary[t] = B;
}

// FP64 helpers from the FP32 vertices: the reference's helper formulas
// (dSim3/src/spinSystem.cpp:612-648) evaluated in double, in the order the
// FP64 oracle evaluates them
__global__ void k_tri64(uint32_t nT, const float* __restrict__ V, const uint32_t* __restrict__ trgls,
                        Tri64* out) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nT) return;
    const uint32_t ia = trgls[3 * t], ib = trgls[3 * t + 1], ic = trgls[3 * t + 2];
    const double ax = V[3 * ia], ay = V[3 * ia + 1], az = V[3 * ia + 2];
    const double bx = V[3 * ib], by = V[3 * ib + 1], bz = V[3 * ib + 2];
    const double cx = V[3 * ic], cy = V[3 * ic + 1], cz = V[3 * ic + 2];
    const double nx = (by - ay) * (cz - az) - (bz - az) * (cy - ay);
    const double ny = (bz - az) * (cx - ax) - (bx - ax) * (cz - az);
    const double nz = (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
    const double len = sqrt(nx * nx + ny * ny + nz * nz);
    Tri64 r;
    r.nx = nx / len; r.ny = ny / len; r.nz = nz / len;
    r.p1x = ax; r.p1y = ay; r.p1z = az;
    r.ux = cx - ax; r.uy = cy - ay; r.uz = cz - az;
    r.vx = bx - ax; r.vy = by - ay; r.vz = bz - az;
    r.uv = r.ux * r.vx + r.uy * r.vy + r.uz * r.vz;
    r.uu = r.ux * r.ux + r.uy * r.uy + r.uz * r.uz;
    r.vv = r.vx * r.vx + r.vy * r.vy + r.vz * r.vz;
    r.pad = 0.0;
    out[t] = r;
}

// records from the reference's own helper arrays (compat path: helpers[12T],
// triInfo[3T] = {fiber, membrane, firstVertex}, vertices[3V])
__global__ void k_records_from_helpers(uint32_t nT, const float* __restrict__ V,
                                       const float* __restrict__ H,
                                       const uint32_t* __restrict__ triInfo, TriPlane* plane,
                                       TriBary* bary) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nT) return;
    const float* h = H + 12 * (size_t)t;
    uint32_t p1 = triInfo[3 * t + 2];
    TriPlane P; TriBary B;
    P.nx = h[0]; P.ny = h[1]; P.nz = h[2];
    P.p1x = V[3 * p1]; P.p1y = V[3 * p1 + 1]; P.p1z = V[3 * p1 + 2];
    P.vv = h[11];
    P.info = pack_info(triInfo[3 * t + 1], triInfo[3 * t]);
    B.ux = h[3]; B.uy = h[4]; B.uz = h[5];
    B.vx = h[6]; B.vy = h[7]; B.vz = h[8];
    B.uv = h[9]; B.uu = h[10];
    plane[t] = P;
    bary[t] = B;
}

// ------------------------------------------------------------------------
// Exact grid membership (populateCubes)
// ------------------------------------------------------------------------
struct f3 { float x, y, z; };
__device__ __forceinline__ f3 mk3(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ f3 sub3(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

__device__ __forceinline__ bool point_in_cube(f3 p, f3 mn, f3 mx) {
    return ((p.x <= mx.x) && (p.x >= mn.x)) && ((p.y <= mx.y) && (p.y >= mn.y)) &&
           ((p.z <= mx.z) && (p.z >= mn.z));
}

// rayTriangleIntersect, dSim3/src/spinSystem.cpp:1360-1379
__device__ bool ray_tri(f3 rp1, f3 rp2, f3 tp1, f3 tp2, f3 tp3) {
    f3 u = sub3(tp2, tp1);
    f3 v = sub3(tp3, tp1);
    f3 n = mk3(u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x);
    float nlength = sqrtf(n.x * n.x + n.y * n.y + n.z * n.z);
    float s = 2.0f, t = 2.0f;
    n.x = n.x / nlength; n.y = n.y / nlength; n.z = n.z / nlength;
    float r = dot3(n, sub3(tp1, rp1)) / dot3(n, sub3(rp2, rp1));
    if ((0.0f < r) & (r < 1.0f)) {
        f3 d = sub3(rp2, rp1);
        f3 w = sub3(mk3(rp1.x + d.x * r, rp1.y + d.y * r, rp1.z + d.z * r), tp1);
        float uv = dot3(u, v), wv = dot3(w, v), vv = dot3(v, v), wu = dot3(w, u), uu = dot3(u, u);
        s = (uv * wv - vv * wu) / (uv * uv - uu * vv);
        t = (uv * wu - uu * wv) / (uv * uv - uu * vv);
    }
    return (s >= 0.0f) && (t >= 0.0f) && (s + t <= 1.0f);
}

// corner b: bit0 = x max, bit1 = y max, bit2 = z max
__device__ __forceinline__ f3 corner(f3 mn, f3 mx, int b) {
    return mk3((b & 1) ? mx.x : mn.x, (b & 2) ? mx.y : mn.y, (b & 4) ? mx.z : mn.z);
}
// cube edges and face triangles in the argument order of spinSystem.cpp:1192-1245
__constant__ unsigned char c_edges[12][2] = {{0, 1}, {0, 2}, {0, 4}, {6, 2}, {6, 4}, {6, 7},
                                             {3, 2}, {3, 1}, {3, 7}, {5, 7}, {5, 1}, {5, 4}};
__constant__ unsigned char c_faces[12][3] = {{0, 1, 2}, {0, 4, 2}, {0, 4, 1}, {6, 2, 4},
                                             {6, 2, 7}, {6, 4, 7}, {3, 2, 1}, {3, 7, 1},
                                             {3, 7, 2}, {5, 4, 7}, {5, 1, 7}, {5, 4, 1}};

__device__ bool tri_cube_overlap(f3 p1, f3 p2, f3 p3, f3 cmin, f3 cmax) {
    if (point_in_cube(p1, cmin, cmax) || point_in_cube(p2, cmin, cmax) || point_in_cube(p3, cmin, cmax))
        return true;
    for (int e = 0; e < 12; e++)
        if (ray_tri(corner(cmin, cmax, c_edges[e][0]), corner(cmin, cmax, c_edges[e][1]), p1, p2, p3))
            return true;
    f3 a[3] = {p1, p1, p2}, b[3] = {p2, p3, p3};
    for (int k = 0; k < 3; k++)
        for (int f = 0; f < 12; f++)
            if (ray_tri(a[k], b[k], corner(cmin, cmax, c_faces[f][0]), corner(cmin, cmax, c_faces[f][1]),
                        corner(cmin, cmax, c_faces[f][2])))
                return true;
    return false;
}

// pass 1 (count) and pass 2 (fill) of the grid build, one thread per triangle
template <bool FILL>
__global__ void k_tri_cells(uint32_t nT, const float* __restrict__ V,
                            const uint32_t* __restrict__ trgls, uint32_t n, float L,
                            uint32_t* counter, const uint32_t* __restrict__ start,
                            uint32_t* cell_tri) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nT) return;
    uint32_t i1 = trgls[3 * t], i2 = trgls[3 * t + 1], i3 = trgls[3 * t + 2];
    f3 p1 = mk3(V[3 * i1], V[3 * i1 + 1], V[3 * i1 + 2]);
    f3 p2 = mk3(V[3 * i2], V[3 * i2 + 1], V[3 * i2 + 2]);
    f3 p3 = mk3(V[3 * i3], V[3 * i3 + 1], V[3 * i3 + 2]);
    f3 mn = p1, mx = p1;
    if (p2.x < mn.x) mn.x = p2.x; if (p3.x < mn.x) mn.x = p3.x;
    if (p2.y < mn.y) mn.y = p2.y; if (p3.y < mn.y) mn.y = p3.y;
    if (p2.z < mn.z) mn.z = p2.z; if (p3.z < mn.z) mn.z = p3.z;
    if (p2.x > mx.x) mx.x = p2.x; if (p3.x > mx.x) mx.x = p3.x;
    if (p2.y > mx.y) mx.y = p2.y; if (p3.y > mx.y) mx.y = p3.y;
    if (p2.z > mx.z) mx.z = p2.z; if (p3.z > mx.z) mx.z = p3.z;
    uint32_t x0 = cube_coord(mn.x, L, n), y0 = cube_coord(mn.y, L, n), z0 = cube_coord(mn.z, L, n);
    uint32_t x1 = cube_coord(mx.x, L, n), y1 = cube_coord(mx.y, L, n), z1 = cube_coord(mx.z, L, n);
    for (uint32_t xc = x0; xc <= x1; xc++)
        for (uint32_t yc = y0; yc <= y1; yc++)
            for (uint32_t zc = z0; zc <= z1; zc++) {
                uint32_t cube = n * n * zc + n * yc + xc;
                f3 cmin = mk3(-1.0f + (float)xc * L, -1.0f + (float)yc * L, -1.0f + (float)zc * L);
                f3 cmax = mk3(-1.0f + (float)(xc + 1) * L, -1.0f + (float)(yc + 1) * L,
                              -1.0f + (float)(zc + 1) * L);
                if (tri_cube_overlap(p1, p2, p3, cmin, cmax)) {
                    uint32_t slot = atomicAdd(counter + cube, 1u);
                    if (FILL) cell_tri[start[cube] + slot] = t;
                }
            }
}

// ascending triangle order inside each cell (the reference's list order)
__global__ void k_sort_cells(uint32_t ncells, const uint32_t* __restrict__ start, uint32_t* cell_tri) {
    uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    uint32_t b = start[c], e = start[c + 1];
    for (uint32_t i = b + 1; i < e; i++) {
        uint32_t v = cell_tri[i];
        uint32_t j = i;
        while (j > b && cell_tri[j - 1] > v) { cell_tri[j] = cell_tri[j - 1]; j--; }
        cell_tri[j] = v;
    }
}

// dense reference grid [cell][maxTPC] -> CSR lists (order kept).  Entries
// that name a triangle >= nT, or cells holding more than maxTPC entries, set
// kStatusBadCell and are replaced by triangle 0's index only as a placeholder
// (the caller refuses to run on such a grid).
__global__ void k_dense_to_csr(uint32_t ncells, uint32_t maxTPC, uint32_t nT,
                               const uint32_t* __restrict__ counter,
                               const uint32_t* __restrict__ dense, const uint32_t* __restrict__ start,
                               uint32_t* cell_tri, uint32_t* status) {
    uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    uint32_t k = counter[c], s = start[c];
    if (k > maxTPC) { atomicOr(status, kStatusBadCell); k = maxTPC; }
    for (uint32_t j = 0; j < k; j++) {
        uint32_t t = dense[(size_t)c * maxTPC + j];
        if (t >= nT) { atomicOr(status, kStatusBadCell); t = 0; }
        cell_tri[s + j] = t;
    }
}

// ------------------------------------------------------------------------
// Host launchers
// ------------------------------------------------------------------------
int launch_records_from_mesh(uint32_t nT, const float* V, const uint32_t* trgls,
                             const uint32_t* membrane, const uint32_t* fiber, TriPlane* plane,
                             TriBary* bary, cudaStream_t st) {
    if (nT == 0) return kOk;
    k_records_from_mesh<<<(nT + 255) / 256, 256, 0, st>>>(nT, V, trgls, membrane, fiber, plane, bary);
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}

// every triangle's reference cells: one thread per cell appends the cell to
// each of its triangles' records (order within a record is irrelevant)
__global__ void k_tri_cell_lists(uint32_t ncells, const uint32_t* __restrict__ cell_start,
                                 const uint32_t* __restrict__ cell_tri, uint32_t* count, uint4* out) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    for (uint32_t k = cell_start[c]; k < cell_start[c + 1]; k++) {
        const uint32_t t = cell_tri[k];
        const uint32_t slot = atomicAdd(count + t, 1u);
        if (slot < 4) reinterpret_cast<uint32_t*>(out + t)[slot] = c;
    }
}
__global__ void k_tri_cell_many(uint32_t nT, const uint32_t* __restrict__ count, uint4* out) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nT && count[t] > 4) out[t] = make_uint4(kCellMany, kCellMany, kCellMany, kCellMany);
}

int launch_tri_cell_lists(uint32_t ncells, uint32_t nT, const uint32_t* cell_start, const uint32_t* cell_tri,
                          uint32_t* count, uint4* out, cudaStream_t st) {
    if (nT == 0) return kOk;
    DSIM_CUDA_TRY(cudaMemsetAsync(count, 0, (size_t)nT * 4, st));
    DSIM_CUDA_TRY(cudaMemsetAsync(out, 0xFF, (size_t)nT * sizeof(uint4), st));
    k_tri_cell_lists<<<(ncells + 255) / 256, 256, 0, st>>>(ncells, cell_start, cell_tri, count, out);
    k_tri_cell_many<<<(nT + 255) / 256, 256, 0, st>>>(nT, count, out);
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}

int launch_tri64(uint32_t nT, const float* V, const uint32_t* trgls, Tri64* out, cudaStream_t st) {
    if (nT == 0) return kOk;
    k_tri64<<<(nT + 255) / 256, 256, 0, st>>>(nT, V, trgls, out);
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}

int launch_records_from_helpers(uint32_t nT, const float* V, const float* H, const uint32_t* triInfo,
                                TriPlane* plane, TriBary* bary, cudaStream_t st) {
    if (nT == 0) return kOk;
    k_records_from_helpers<<<(nT + 255) / 256, 256, 0, st>>>(nT, V, H, triInfo, plane, bary);
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}

int launch_tri_cells(bool fill, uint32_t nT, const float* V, const uint32_t* trgls, uint32_t n,
                     float L, uint32_t* counter, const uint32_t* start, uint32_t* cell_tri,
                     cudaStream_t st) {
    if (nT == 0) return kOk;
    if (fill)
        k_tri_cells<true><<<(nT + 127) / 128, 128, 0, st>>>(nT, V, trgls, n, L, counter, start, cell_tri);
    else
        k_tri_cells<false><<<(nT + 127) / 128, 128, 0, st>>>(nT, V, trgls, n, L, counter, start, cell_tri);
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}

int launch_sort_cells(uint32_t ncells, const uint32_t* start, uint32_t* cell_tri, cudaStream_t st) {
    k_sort_cells<<<(ncells + 255) / 256, 256, 0, st>>>(ncells, start, cell_tri);
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}

int launch_dense_to_csr(uint32_t ncells, uint32_t maxTPC, uint32_t nT, const uint32_t* counter,
                        const uint32_t* dense, const uint32_t* start, uint32_t* cell_tri,
                        uint32_t* status, cudaStream_t st) {
    k_dense_to_csr<<<(ncells + 255) / 256, 256, 0, st>>>(ncells, maxTPC, nT, counter, dense, start,
                                                          cell_tri, status);
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}

}  // namespace dsim

// ---------------------------------------------------------------------------
// The step kernels' draws, exposed for testing the generator on its own.
// ---------------------------------------------------------------------------
namespace dsim {
__global__ void k_rng_draws(uint32_t k0, uint32_t k1, uint32_t spin0, uint64_t step,
                            uint32_t stream, uint32_t n, uint4* raw, float4* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    u32x4 c = {spin0 + i, (uint32_t)step, (uint32_t)(step >> 32), stream};
    u32x4 r = philox4x32_10(c, k0, k1);
    raw[i] = make_uint4(r.x, r.y, r.z, r.w);
    Draw d = philox_draw(spin0 + i, step, stream, k0, k1);
    out[i] = make_float4(d.nx, d.ny, d.nz, d.u);
}

int launch_rng_draws(uint64_t seed, uint32_t spin0, uint64_t step, uint32_t stream, uint32_t n,
                     uint32_t* raw, float* out, cudaStream_t st) {
    if (n == 0) return kOk;
    k_rng_draws<<<(n + 255) / 256, 256, 0, st>>>((uint32_t)seed, (uint32_t)(seed >> 32), spin0, step,
                                                 stream, n, reinterpret_cast<uint4*>(raw),
                                                 reinterpret_cast<float4*>(out));
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}
}  // namespace dsim
