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
