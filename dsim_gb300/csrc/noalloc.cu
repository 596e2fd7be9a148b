// noalloc.cu -- ensemble signal over the reference's spin arrays without any
// device allocation.
//
// dsim_signal works in scratch owned by a dsim_spins object.  Some callers
// cannot allocate device memory at the moment they need the signal:
//  * a host that links only the reference's C-ABI (dSim3/src/spinSystem.cuh)
//    owns every device buffer itself and has no engine object to lend scratch;
//  * a serving loop that has handed all free HBM to admitted jobs, where a
//    new allocation would fail or evict a job;
//  * code between the kernels of a pipelined step that must not stall other
//    streams, which cudaMalloc and cudaFree can do by synchronising the device.
// This entry point therefore takes its scratch from a fixed array compiled
// into the library and calls no allocator (no cudaMalloc/cudaFree, no library
// that allocates).
//
// Scratch: one partial record of 15 doubles per block of 2048 spins, at most
// 8192 records (983,040 bytes), so N is limited to 16,777,216 spins; larger N
// is rejected with DSIM_ETOOLARGE before anything is launched.  Nothing in the
// scratch has to start at zero: the partial pass writes every record the final
// pass reads, in the same call.  The array is shared by every call on a
// device, so calls that could overlap (different streams, or host threads
// without ordering) race on it; callers serialise them, e.g. on one stream.
//
// Setup: every call looks up the array's device address on the current device
// with cudaGetSymbolAddress (it allocates nothing), so an address never
// outlives a cudaDeviceReset that reloads the module.  The first call on a
// device also loads the module there: make it before any stream capture.
#include <cstdint>

#pragma GCC visibility push(default)
#include "../../include/dsim.h"
#pragma GCC visibility pop
#include "common.cuh"
#include "engine.h"

namespace dsim {

static constexpr uint32_t kNaVals = 15;            // (X, Y, n) x (total + 4 compartments)
static constexpr uint32_t kNaSpinsPerBlock = 2048;  // 256 threads x 8 spins per partial record
static constexpr uint32_t kNaMaxBlocks = 8192;
static constexpr uint32_t kNaMaxSpins = kNaSpinsPerBlock * kNaMaxBlocks;
static __device__ __align__(256) double g_signal_scratch[kNaMaxBlocks * kNaVals];

// device address of the scratch array on the current device
static int scratch_for_current_device(double** out) {
    double* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_signal_scratch);
    if (e != cudaSuccess || !ptr) {
        int dev = -1;
        cudaGetDevice(&dev);
        set_last_error(kErrCuda, "dsim_signal_noalloc: cudaGetSymbolAddress of the scratch on device %d: %s", dev,
                       cudaGetErrorString(e));
        return kErrCuda;
    }
    *out = ptr;
    return kOk;
}

}  // namespace dsim

using namespace dsim;

extern "C" int dsim_signal_noalloc(const float* pos, const void* spinRecords, uint32_t N, int layout,
                                   double region, double* out, void* stream) {
    if (layout != DSIM_SIGNAL_DSIM3 && layout != DSIM_SIGNAL_DSIM2) {
        set_last_error(kErrInvalid, "dsim_signal_noalloc: layout %d is neither dSim3 (1) nor dSim2 (2)", layout);
        return kErrInvalid;
    }
    if (!out || (N > 0 && !pos) || (N > 0 && layout == DSIM_SIGNAL_DSIM3 && !spinRecords)) {
        set_last_error(kErrInvalid, "dsim_signal_noalloc: null argument");
        return kErrInvalid;
    }
    if (N > kNaMaxSpins) {
        set_last_error(kErrTooLarge, "dsim_signal_noalloc: %u spins exceed the fixed scratch's limit of %u",
                       N, kNaMaxSpins);
        return kErrTooLarge;
    }
    double* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc != kOk) return rc;
    SpinsDev S{};
    S.x = const_cast<float*>(pos);
    S.meta = const_cast<uint32_t*>(static_cast<const uint32_t*>(spinRecords));
    S.mag = nullptr;  // dSim2 arrays carry no magnitude (1.0)
    S.N = N;
    int nb = (int)((N + kNaSpinsPerBlock - 1) / kNaSpinsPerBlock);
    return launch_signal_blocks(S, layout == DSIM_SIGNAL_DSIM3 ? kLayoutAoS : 2, region, scratch,
                                nb, out, static_cast<cudaStream_t>(stream));
}
