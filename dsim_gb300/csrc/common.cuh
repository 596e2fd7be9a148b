// common.cuh -- shared device/host definitions of the GB300 dSim engine.
//
// Everything that decides a spin's trajectory is compiled with -fmad=false
// and IEEE division/square root, so each float operation rounds exactly like
// the reference's CPU build (rfdougherty/dSim, dSim3/src/spinKernelCpu.cpp and
// dSim2/src/spinKernelCpu.cpp); the replay tests compare bit for bit.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace dsim {

// ---- status codes (also the C-ABI return values) ------------------------
enum Status : int {
    kOk = 0,
    kErrInvalid = -1,       // bad argument
    kErrCuda = -2,          // CUDA runtime error
    kErrFile = -3,          // cannot open / parse an input file
    kErrFormat = -4,        // file parsed but rejected (as the reference does)
    kErrNoMem = -5,         // device allocation failed
    kErrTooLarge = -6,      // request above a stated limit
    kErrGridOverflow = -7,  // a grid cell exceeds its capacity (dSim2 build())
};

// device-side status bits written by kernels into a status word
enum StatusBits : uint32_t {
    kStatusSubsegCap = 1u,   // a spin hit the sub-segment cap in one step
    kStatusBadCell = 2u,     // a cell index fell outside the grid (never expected)
    kStatusParityOverflow = 4u,  // compartment search: more than 32 membranes on one line
    kStatusUnresolved = 8u,      // compartment search: every line and position was ambiguous
    kStatusStageTimeout = 16u,   // a bulk-copy wait ran out (the warp stopped; its spins are stale)
};

// ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) -------------------
struct u32x4 { uint32_t x, y, z, w; };

__host__ __device__ __forceinline__ void mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
#ifdef __CUDA_ARCH__
    lo = a * b;
    hi = __umulhi(a, b);
#else
    uint64_t p = (uint64_t)a * b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
#endif
}

__host__ __device__ __forceinline__ u32x4 philox4x32_10(u32x4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(0xD2511F53u, c.x, hi0, lo0);
        mulhilo32(0xCD9E8D57u, c.z, hi1, lo1);
        u32x4 n;
        n.x = hi1 ^ c.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ c.w ^ k1;
        n.w = lo0;
        c = n;
    }
    return c;
}

#if defined(__CUDACC__)
// floorf(t) for |t| < 2^22 on the FP32 pipe, without a rounding or
// conversion instruction: adding and subtracting 1.5 * 2^23 rounds t to an
// integer (the sum's ulp is 1), and a step down undoes rounding up.  The same
// value as floorf (a zero result is +0).
__device__ __forceinline__ float floor_small(float t) {
    const float r = __fsub_rn(__fadd_rn(t, 12582912.0f), 12582912.0f);
    return r > t ? __fsub_rn(r, 1.0f) : r;
}
// (uint32_t)f for an integer-valued f in [0, 2^23): f + 2^23 holds f in its
// significand.
__device__ __forceinline__ uint32_t uint_small(float f) {
    return __float_as_uint(__fadd_rn(f, 8388608.0f)) - 0x4B000000u;
}
#endif

// One step's draws for one spin: counter = (spin, step lo, step hi, stream),
// key = 64-bit job seed.  The four words map to the reference's myRandn
// layout (dSim3/src/spinKernelCpu.cpp:53-63): Box-Muller on (u1,u2) gives
// n.x, n.y; on (u3,u4) gives n.z; u4 is also the permeation uniform u.
struct Draw { float nx, ny, nz, u; };

#if defined(__CUDACC__)
// Box-Muller radius argument in (0, 1]: x * 2^-32 + 2^-33 (never 0, so the
// logarithm is finite; tails reach 6.8 sigma).
__device__ __forceinline__ float u01_log(uint32_t x) {
    return __fmaf_rn((float)x, 2.3283064365386963e-10f, 1.1641532182693481e-10f);
}
// Angle argument in [0, 1) with 24-bit resolution (exact).
__device__ __forceinline__ float u01_angle(uint32_t x) {
    return (float)(x >> 8) * 5.9604644775390625e-08f;
}
// Uniform in (0, 1] with 24-bit resolution (exact), like the reference's
// ((float)r + 1) / 2^32 range.
__device__ __forceinline__ float u01_half_open(uint32_t x) {
    return (float)((x >> 8) + 1u) * 5.9604644775390625e-08f;
}

__device__ __forceinline__ Draw philox_draw(uint32_t spin, uint64_t step, uint32_t stream,
                                            uint32_t k0, uint32_t k1) {
    u32x4 c = {spin, (uint32_t)step, (uint32_t)(step >> 32), stream};
    u32x4 r = philox4x32_10(c, k0, k1);
    float u1 = u01_log(r.x), u2 = u01_angle(r.y), u3 = u01_log(r.z), u4 = u01_half_open(r.w);
    float rad1 = sqrtf(-2.0f * logf(u1));
    float rad2 = sqrtf(-2.0f * logf(u3));
    float s1, c1, c2;
    sincospif(2.0f * u2, &s1, &c1);
    c2 = cospif(2.0f * u4);
    Draw d;
    d.nx = rad1 * c1;
    d.ny = rad1 * s1;
    d.nz = rad2 * c2;
    d.u = u4;
    return d;
}
#endif  // __CUDACC__

// ---- geometry records held in HBM for the mesh path ---------------------
// Per triangle, the reference's helper values (dSim3/src/spinSystem.cpp:612-648)
// regrouped for the two stages of triCollDetect: the plane test needs the
// normal and the first vertex (32 B, one sector); the barycentric test needs
// u, v and the three dot products (second 32-B record, read on plane hits only).
struct __align__(16) TriPlane {
    float nx, ny, nz, p1x;
    float p1y, p1z, vv;
    uint32_t info;  // membrane type (bits 0-1) | fiber index << 2
};
struct __align__(16) TriBary {
    float ux, uy, uz, vx;
    float vy, vz, uv, uu;
};

__host__ __device__ __forceinline__ uint32_t pack_info(uint32_t membrane, uint32_t fiber) {
    return (membrane & 3u) | (fiber << 2);
}

// Region of a dSim2 spin (0 core, 1 myelin, 2 outside) from words 2 and 3 of
// its seed record.  The engine stores imo + 1 in word 2.  The reference's
// assignSeeds (dSim2/src/spinSystem.cpp:1129-1151) leaves word 2 at 0 and
// puts the nearest fiber in word 3 for a spin inside a fiber, UINT_MAX for one
// outside; such a record reads as core or outside.  A word 2 above 3 gives a
// region above 2: the step treats it as outside, and the signal sums region 3
// in its own slot and any higher region in the total only.
__host__ __device__ __forceinline__ uint32_t dsim2_region(uint32_t w2, uint32_t w3) {
    return (w2 == 0u) ? ((w3 != 0xFFFFFFFFu) ? 0u : 2u) : (w2 - 1u);
}

}  // namespace dsim

#define DSIM_CUDA_TRY(expr)                                  \
    do {                                                     \
        cudaError_t _e = (expr);                             \
        if (_e != cudaSuccess) {                             \
            dsim::set_last_cuda_error(_e, #expr, __FILE__, __LINE__); \
            return dsim::kErrCuda;                           \
        }                                                    \
    } while (0)

namespace dsim {
void set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line);
void set_last_error(int code, const char* fmt, ...);
}
