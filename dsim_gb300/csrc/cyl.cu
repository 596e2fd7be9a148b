// cyl.cu -- infinite-cylinder (fiber) substrate: the random-walk step with the
// reference's endpoint-in-disk membrane test.
//
// Reference (rfdougherty/dSim): cpuIntegrate dSim2/src/spinKernelCpu.cpp:312-641,
// distToCenterSq :71-82, calcCubePos/calcCubeHash dSim2/src/spinSystem.cpp:413-433.
// A step that would cross a membrane is rejected (the spin stays at its old
// position) unless the permeation draw lets it through; a spin outside all
// fibers is tested against the fibers listed in the cell of its new position,
// followed by the reference's second "bounced into another fiber" pass.
// Compiled with -fmad=false so replayed trajectories match the CPU bit for bit.
#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>
#include "common.cuh"
#include "cyl_common.cuh"
#include "engine.h"

namespace dsim {

// Default fine filter grid size for a reference grid of n cells per axis of
// edge L and largest fiber radius maxR: fine cells about half the largest
// radius across, at most 16 per grid-cell edge and 2^22 fine cells in all;
// 0 when that leaves fewer than 2.
uint32_t cyl_fine_size(uint32_t n, float L, double maxR) {
    if (!(maxR > 0.0) || n == 0) return 0;
    uint32_t k = (uint32_t)std::min(16.0, std::ceil(2.0 * (double)L / maxR));
    while (k >= 2 && (uint64_t)(n * k) * (n * k) * (n * k) > (1ull << 22)) k--;
    return k >= 2 ? k : 0;
}

// The fine lists on the host: start[(n k)^3 + 1] offsets, and per entry its
// list position and fiber record.  Every listed fiber index must be < nF.
int cyl_fine_lists(const float* fiberPos, uint32_t nF, uint32_t n, uint32_t maxFPC, float cubeLength,
                   const uint32_t* cubeCounter, const uint32_t* cubes, uint32_t k, std::vector<uint32_t>& start,
                   std::vector<uint32_t>& pos, std::vector<float>& rec) {
    if (k < 2 || n == 0 || (uint64_t)(n * k) * (n * k) * (n * k) > (1ull << 24)) {
        set_last_error(kErrTooLarge, "cylinder fine grid: (%u x %u)^3 cells, limit 2^24 and k >= 2", n, k);
        return kErrTooLarge;
    }
    const uint32_t nk = n * k;
    const size_t nfine = (size_t)nk * nk * nk;
    const double L = (double)cubeLength;
    const double Lf = L / k, eps = 1e-5, inf = std::numeric_limits<double>::infinity();
    start.assign(nfine + 1, 0);
    pos.clear();
    rec.clear();
    for (size_t fc = 0; fc < nfine; fc++) {
        const uint32_t gx = (uint32_t)(fc % nk), gy = (uint32_t)((fc / nk) % nk), gz = (uint32_t)(fc / ((size_t)nk * nk));
        const uint32_t gcoord[3] = {gx, gy, gz};
        double lo[3], hi[3];
        for (int a = 0; a < 3; a++) {
            lo[a] = gcoord[a] == 0 ? -inf : -1.0 + gcoord[a] * Lf - eps;
            hi[a] = gcoord[a] == nk - 1 ? inf : -1.0 + (gcoord[a] + 1) * Lf + eps;
        }
        const size_t cell = ((size_t)(gz / k) * n + gy / k) * n + gx / k;
        if (cubeCounter[cell] > maxFPC) {
            set_last_error(kErrFormat, "cylinder grid: cell %zu lists %u entries, limit %u", cell, cubeCounter[cell], maxFPC);
            return kErrFormat;
        }
        for (uint32_t j = 0; j < cubeCounter[cell]; j++) {
            const uint32_t fi = cubes[cell * maxFPC + j];
            if (fi >= nF) {
                set_last_error(kErrFormat, "cylinder grid: entry names fiber %u of %u", fi, nF);
                return kErrFormat;
            }
            const float* f = &fiberPos[4 * (size_t)fi];
            // the axes of the distance, as the step's distance function picks them
            int a0 = 0, a1 = 2;
            if (f[0] == 2.0f) { a0 = 1; a1 = 2; }
            else if (f[2] == 2.0f) { a0 = 0; a1 = 1; }
            double d2 = 0.0;
            for (int a : {a0, a1}) {
                const double x = (double)f[a];
                const double d = std::max(std::max(lo[a] - x, 0.0), x - hi[a]);
                d2 += d * d;
            }
            if (d2 <= (double)f[3] * (1.0 + 1e-4)) {
                pos.push_back(j);
                for (int q = 0; q < 4; q++) rec.push_back(f[q]);
            }
        }
        start[fc + 1] = (uint32_t)pos.size();
        if (pos.size() > 0xF0000000u) {
            set_last_error(kErrTooLarge, "cylinder fine grid: too many entries");
            return kErrTooLarge;
        }
    }
    return kOk;
}

// ---- the reference's cylinder grid, built on the GPU ----------------------
// addEntities (dSim2/src/spinSystem.cpp:483-745): a fiber is listed in every
// cell of the line of cells along its axis through its centre (the line's
// cells found by stepping a point from -1 + 0.002 by one cell length), and in
// the neighbouring lines that its radius plus a 1.1 halo can reach.  One
// thread per fiber replays that insertion sequence with the same float
// operations; pass 1 counts the entries per cell, pass 2 files each entry with
// its tag (fiber << 10 | insertion index), and a per-cell sort of the tags
// restores the reference's order (fibers in file order, each fiber's lines in
// the order addEntities adds them, repeats kept).
static constexpr uint32_t kCylSeqBits = 10;  // insertion index: at most 5 lines x 100 cells

template <typename Emit>
__device__ void cyl_fiber_insertions(float4 fr, uint32_t n, float L, float H, Emit emit) {
    float fp[3] = {fr.x, fr.y, fr.z};
    int a, f, s;
    if (fp[0] == 2.0f) { a = 0; f = 2; s = 1; }
    else if (fp[2] == 2.0f) { a = 2; f = 0; s = 1; }
    else if (fp[1] == 2.0f) { a = 1; f = 2; s = 0; }
    else return;
    const float start = (float)(-1.0 + 0.002);
    uint32_t seq = 0;
    auto line = [&](float* cp) {
        cp[a] = start;
        for (uint32_t j = 0; j < n; j++) {
            emit(cyl_cell(cp[0], cp[1], cp[2], L, n), seq++);
            cp[a] += L;
        }
    };
    float cp[3] = {fp[0], fp[1], fp[2]};
    line(cp);
    float tp[3] = {fp[0], fp[1], fp[2]};
    tp[a] = start;
    const float inv = 1.0f / L;
    const float cpos_f = floorf((tp[f] + 1.0f) * inv), cpos_s = floorf((tp[s] + 1.0f) * inv);
    const float dfc_f = tp[f] - cpos_f * L;
    const float dfc_s = tp[s] - cpos_s * L;
    if (dfc_f < H) {
        cp[f] -= H;
        if (cp[f] > -1) {
            line(cp);
            if ((cp[s] - L) > -1) { cp[s] -= L; line(cp); cp[s] += L; }
            if ((cp[s] + L) < 1) { cp[s] += L; line(cp); cp[s] -= L; }
        }
        cp[f] += H;
    } else if (dfc_f > (L - H)) {
        cp[f] += H;
        if (cp[f] < 1) {
            line(cp);
            if ((cp[s] - L) > -1) { cp[s] -= L; line(cp); cp[s] += L; }
            if ((cp[s] + L) < 1) { cp[s] += L; line(cp); cp[s] -= L; }
        }
        cp[f] -= H;
    }
    if (dfc_s < H) {
        if ((cp[s] - L) > -1) { cp[s] -= L; line(cp); cp[s] += L; }
    } else if (dfc_s > (L - H)) {
        if ((cp[s] + L) < 1) { cp[s] += L; line(cp); cp[s] -= L; }
    }
}

__global__ void k_cyl_grid_count(const float4* __restrict__ fibers, uint32_t nF, uint32_t n, float L, float H,
                                 uint32_t* counter) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nF) return;
    cyl_fiber_insertions(fibers[i], n, L, H, [&](uint32_t cell, uint32_t) { atomicAdd(counter + cell, 1u); });
}

__global__ void k_cyl_grid_fill(const float4* __restrict__ fibers, uint32_t nF, uint32_t n, float L, float H,
                                uint32_t maxFPC, uint32_t* counter, uint32_t* tags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nF) return;
    cyl_fiber_insertions(fibers[i], n, L, H, [&](uint32_t cell, uint32_t seq) {
        const uint32_t slot = atomicAdd(counter + cell, 1u);
        if (slot < maxFPC) tags[(size_t)cell * maxFPC + slot] = (i << kCylSeqBits) | seq;
    });
}

// per cell: its tags in ascending order become the fiber list; the unused
// slots stay 0 as the reference's memset leaves them
__global__ void k_cyl_grid_order(uint32_t ncells, uint32_t maxFPC, const uint32_t* __restrict__ counter,
                                 uint32_t* tags, uint32_t* cubes) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    uint32_t* t = tags + (size_t)c * maxFPC;
    const uint32_t cnt = min(counter[c], maxFPC);
    for (uint32_t k = 1; k < cnt; k++) {
        const uint32_t v = t[k];
        uint32_t j = k;
        while (j > 0 && t[j - 1] > v) { t[j] = t[j - 1]; j--; }
        t[j] = v;
    }
    uint32_t* out = cubes + (size_t)c * maxFPC;
    for (uint32_t k = 0; k < maxFPC; k++) out[k] = k < cnt ? (t[k] >> kCylSeqBits) : 0u;
}

// each listed entry's fiber record beside it (the step reads one record per entry)
__global__ void k_cyl_grid_inline(size_t slots, uint32_t maxFPC, const uint32_t* __restrict__ counter,
                                  const uint32_t* __restrict__ cubes, const float4* __restrict__ fibers,
                                  float4* cubeF) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= slots) return;
    const uint32_t cell = (uint32_t)(k / maxFPC), j = (uint32_t)(k % maxFPC);
    cubeF[k] = j < counter[cell] ? fibers[cubes[k]] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

int build_cyl_grid_gpu(const float4* fibers, uint32_t nF, uint32_t n, uint32_t maxFPC, float L, float maxR,
                       uint32_t* counter, uint32_t* cubes, float4* cubeF, uint32_t* maxCount, cudaStream_t st) {
    if (nF >= (1u << (32 - kCylSeqBits)) || n > 100) {
        set_last_error(kErrTooLarge, "cylinder grid: %u fibers or %u cells per axis above the build's limits", nF, n);
        return kErrTooLarge;
    }
    const float H = 1.1f * maxR;
    const uint32_t ncells = n * n * n;
    const size_t slots = (size_t)ncells * maxFPC;
    DSIM_CUDA_TRY(cudaMemsetAsync(counter, 0, (size_t)ncells * 4, st));
    const uint32_t fb = (nF + 127) / 128;
    if (nF) k_cyl_grid_count<<<fb, 128, 0, st>>>(fibers, nF, n, L, H, counter);
    DSIM_CUDA_TRY(cudaGetLastError());
    std::vector<uint32_t> cnt(ncells);
    DSIM_CUDA_TRY(cudaMemcpyAsync(cnt.data(), counter, (size_t)ncells * 4, cudaMemcpyDeviceToHost, st));
    DSIM_CUDA_TRY(cudaStreamSynchronize(st));
    uint32_t mx = 0;
    for (uint32_t v : cnt) mx = std::max(mx, v);
    *maxCount = mx;
    if (mx > maxFPC) {
        set_last_error(kErrGridOverflow, "cylinder grid: %u fibers in one cell, limit %u (build() fails)", mx, maxFPC);
        return kErrGridOverflow;
    }
    uint32_t* tags = nullptr;
    DSIM_CUDA_TRY(cudaMalloc(&tags, std::max<size_t>(1, slots) * 4));
    cudaError_t e = cudaMemsetAsync(counter, 0, (size_t)ncells * 4, st);
    if (e == cudaSuccess && nF) {
        k_cyl_grid_fill<<<fb, 128, 0, st>>>(fibers, nF, n, L, H, maxFPC, counter, tags);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_cyl_grid_order<<<(ncells + 127) / 128, 128, 0, st>>>(ncells, maxFPC, counter, tags, cubes);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && cubeF && slots) {
        k_cyl_grid_inline<<<(unsigned)((slots + 255) / 256), 256, 0, st>>>(slots, maxFPC, counter, cubes, fibers,
                                                                          cubeF);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(tags);
    if (e != cudaSuccess) { set_last_cuda_error(e, "cylinder grid build", __FILE__, __LINE__); return kErrCuda; }
    return kOk;
}

template <int RNG>
__global__ void __launch_bounds__(256) k_cyl_step(CylDev g, CylStepArgs a, CylSpinsDev S) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.N) return;
    float4 P = S.pos[i];
    uint4 sd4 = reinterpret_cast<const uint4*>(S.seed4)[i];
    float x = P.x, y = P.y, z = P.z, phase = P.w;
    float mag = S.mag ? S.mag[i] : 1.0f;
    uint32_t nearest = sd4.w;
    uint32_t imo = dsim2_region(sd4.z, nearest);
    if (imo < 2 && nearest >= g.nF) imo = 2;  // no valid fiber: treat as outside
    uint32_t nrej = 0, nperm = 0, status = 0;
    uint32_t k0 = a.key0, k1 = a.key1;
    if (RNG == kRngPhiloxPerSpinKey) { k0 = sd4.x; k1 = sd4.y; }
    const float perm = a.perm, inR = a.inRadPropSq;
    for (uint32_t it = 0; it < a.iterations; it++) {
        Draw d;
        if (RNG == kRngReplay) {
            float4 q = __ldg(a.draws + (size_t)it * S.N + i);
            d.nx = q.x; d.ny = q.y; d.nz = q.z; d.u = q.w;
        } else {
            d = philox_draw(a.spinBase + i, a.step0 + it, a.stream, k0, k1);
        }
        float ox = x, oy = y, oz = z;
        float sdv = (imo == 0) ? a.intraSd : ((imo == 1) ? a.myelinSd : a.extraSd);
        float px = x + d.nx * sdv, py = y + d.ny * sdv, pz = z + d.nz * sdv;
        cyl_membranes(g, ox, oy, oz, px, py, pz, d.u, perm, inR, imo, nearest, nrej, nperm, status);
        if (px > a.clampHi) px = a.clampHi; else if (px < a.clampLo) px = a.clampLo;
        if (py > a.clampHi) py = a.clampHi; else if (py < a.clampLo) py = a.clampLo;
        if (pz > a.clampHi) pz = a.clampHi; else if (pz < a.clampLo) pz = a.clampLo;
        x = px; y = py; z = pz;
        float T2 = (imo == 0) ? a.T2fiber : ((imo == 1) ? a.T2myelin : a.T2outside);
        mag += -mag / T2 * a.dt;
        float gx = a.gx, gy = a.gy, gz = a.gz;
        if (a.grad) { float4 G = __ldg(a.grad + it); gx = G.x; gy = G.y; gz = G.z; }
        phase += (gx * x + gy * y + gz * z) * a.pc;
    }
    S.pos[i] = make_float4(x, y, z, phase);
    if (S.mag) S.mag[i] = mag;
    uint4 o4 = sd4;
    o4.z = imo + 1u;
    o4.w = nearest;
    if (RNG == kRngPhiloxPerSpinKey) {
        u32x4 nk = philox4x32_10({i, a.iterations, 0xFFFFFFFFu, 0x5EEDu}, k0, k1);
        o4.x = nk.x; o4.y = nk.y;
    }
    reinterpret_cast<uint4*>(S.seed4)[i] = o4;
    if (a.counts) { a.counts[2 * i] += nrej; a.counts[2 * i + 1] += nperm; }
    if (status) atomicOr(a.status, status);
}

int launch_cyl_step(const CylDev& g, const CylStepArgs& a, const CylSpinsDev& S, int rng,
                    cudaStream_t st) {
    if (S.N == 0 || a.iterations == 0) return kOk;
    dim3 block(128), grid((S.N + 127) / 128);
    if (rng == kRngReplay) k_cyl_step<kRngReplay><<<grid, block, 0, st>>>(g, a, S);
    else if (rng == kRngPhilox) k_cyl_step<kRngPhilox><<<grid, block, 0, st>>>(g, a, S);
    else k_cyl_step<kRngPhiloxPerSpinKey><<<grid, block, 0, st>>>(g, a, S);
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}

}  // namespace dsim
