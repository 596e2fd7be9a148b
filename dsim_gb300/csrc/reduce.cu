// reduce.cu -- ensemble MR signal on the device in FP64.
//
// Reference: SpinSystem::getMrSignal(double[]) dSim3/src/spinSystem.cpp:1452-1500
// (sum of m*cos(phi), m*sin(phi) per compartment, S = |X + iY| / n) and the
// dSim2 variant dSim2/src/spinSystem.cpp:944-978 (spins within +-0.8 only).
// The reference copies every spin to the host for this; here each block
// reduces its spins in double precision into a partial record and one block
// adds the partials in a fixed order (deterministic result).
#include "common.cuh"
#include "engine.h"

namespace dsim {

static constexpr int kRedThreads = 256;
static constexpr int kRedBlocks = 608;  // 4 x 152 SMs
static constexpr int kRedVals = 15;     // (X, Y, n) x (total + 4 compartments)

size_t reduce_scratch_doubles(uint32_t) { return (size_t)kRedBlocks * kRedVals; }

template <int LAYOUT>
__device__ __forceinline__ bool load_sig(const SpinsDev& S, uint32_t i, double region, double& m,
                                         double& ph, uint32_t& comp) {
    float x, y, z;
    // comp above 3 (outside the reference's four compartments) is counted in
    // the total only: the caller sees it as n_total - sum of compartment n.
    if (LAYOUT == kLayoutSoA) {
        x = S.x[i]; y = S.y[i]; z = S.z[i];
        m = S.mag[i]; ph = S.phase[i];
        comp = S.meta[i] & 0xFFu;
    } else if (LAYOUT == kLayoutAoS) {
        x = S.x[3 * i]; y = S.x[3 * i + 1]; z = S.x[3 * i + 2];
        const unsigned char* rec = reinterpret_cast<const unsigned char*>(S.meta) + 12 * (size_t)i;
        m = *reinterpret_cast<const float*>(rec);
        ph = *reinterpret_cast<const float*>(rec + 4);
        comp = rec[8];
    } else {  // cylinder layout: x = float4 {x, y, z, phase}, mag optional
        const float4 p = reinterpret_cast<const float4*>(S.x)[i];
        x = p.x; y = p.y; z = p.z; ph = p.w;
        m = S.mag ? (double)S.mag[i] : 1.0;
        if (S.meta) {
            const uint2 w = reinterpret_cast<const uint2*>(S.meta)[2 * (size_t)i + 1];
            comp = dsim2_region(w.x, w.y);
        } else {
            comp = 0u;
        }
    }
    if (region > 0.0)
        return ((double)x > -region && (double)x < region && (double)y > -region &&
                (double)y < region && (double)z > -region && (double)z < region);
    return true;
}

template <int LAYOUT>
__global__ void __launch_bounds__(kRedThreads) k_signal_partial(SpinsDev S, double region,
                                                                double* partials) {
    double acc[kRedVals];
#pragma unroll
    for (int k = 0; k < kRedVals; k++) acc[k] = 0.0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < S.N; i += gridDim.x * blockDim.x) {
        double m, ph;
        uint32_t comp;
        if (!load_sig<LAYOUT>(S, i, region, m, ph, comp)) continue;
        double s, c;
        sincos(ph, &s, &c);
        double X = m * c, Y = m * s;
        acc[0] += X; acc[1] += Y; acc[2] += 1.0;
#pragma unroll
        for (uint32_t k = 0; k < 4; k++) {
            bool on = (comp == k);
            acc[3 + 3 * k] += on ? X : 0.0;
            acc[4 + 3 * k] += on ? Y : 0.0;
            acc[5 + 3 * k] += on ? 1.0 : 0.0;
        }
    }
    __shared__ double sh[kRedThreads / 32][kRedVals];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < kRedVals; k++) {
        double v = acc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
        if (lane == 0) sh[w][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < kRedVals) {
        double v = 0.0;
        for (int j = 0; j < kRedThreads / 32; j++) v += sh[j][threadIdx.x];
        partials[(size_t)blockIdx.x * kRedVals + threadIdx.x] = v;
    }
}

__global__ void k_signal_final(const double* __restrict__ partials, int nblocks, double* out) {
    int k = threadIdx.x;
    if (k >= kRedVals) return;
    double v = 0.0;
    for (int b = 0; b < nblocks; b++) v += partials[(size_t)b * kRedVals + k];
    out[k] = v;
}

// final pass over nb partial records: warp k adds field k with lane-strided
// partial sums and a shuffle tree (fixed order, deterministic)
__global__ void k_signal_final_warps(const double* __restrict__ partials, int nb, double* out) {
    const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (k >= kRedVals) return;
    double v = 0.0;
    for (int b = lane; b < nb; b += 32) v += partials[(size_t)b * kRedVals + k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    if (lane == 0) out[k] = v;
}

int launch_signal_blocks(const SpinsDev& S, int layout, double region, double* partials, int nb,
                         double* out15, cudaStream_t st) {
    if (nb < 1) nb = 1;
    if (layout == kLayoutSoA) k_signal_partial<kLayoutSoA><<<nb, kRedThreads, 0, st>>>(S, region, partials);
    else if (layout == kLayoutAoS) k_signal_partial<kLayoutAoS><<<nb, kRedThreads, 0, st>>>(S, region, partials);
    else k_signal_partial<2><<<nb, kRedThreads, 0, st>>>(S, region, partials);
    k_signal_final_warps<<<1, 32 * kRedVals, 0, st>>>(partials, nb, out15);
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}

int launch_signal(const SpinsDev& S, int layout, double region, double* partials, double* out15,
                  cudaStream_t st) {
    int nb = kRedBlocks;
    if (layout == kLayoutSoA) k_signal_partial<kLayoutSoA><<<nb, kRedThreads, 0, st>>>(S, region, partials);
    else if (layout == kLayoutAoS) k_signal_partial<kLayoutAoS><<<nb, kRedThreads, 0, st>>>(S, region, partials);
    else k_signal_partial<2><<<nb, kRedThreads, 0, st>>>(S, region, partials);
    k_signal_final<<<1, 32, 0, st>>>(partials, nb, out15);
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}

}  // namespace dsim
