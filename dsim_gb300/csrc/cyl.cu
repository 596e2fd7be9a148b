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
#include "common.cuh"
#include "cyl_common.cuh"
#include "engine.h"

namespace dsim {

template <int RNG>
__global__ void __launch_bounds__(256) k_cyl_step(CylDev g, CylStepArgs a, CylSpinsDev S) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.N) return;
    float4 P = S.pos[i];
    uint4 sd4 = reinterpret_cast<const uint4*>(S.seed4)[i];
    float x = P.x, y = P.y, z = P.z, phase = P.w;
    float mag = S.mag ? S.mag[i] : 1.0f;
    uint32_t nearest = sd4.w;
    uint32_t imo = (sd4.z == 0u) ? ((nearest != 0xFFFFFFFFu) ? 0u : 2u) : (sd4.z - 1u);
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
