// compat2.cu -- libdsim2.so: the dSim2 (cylinder) plugin boundary
// (include/dsim2_abi.h), a drop-in for rfdougherty/dSim dSim2/src/spinSystem.cu.
// integrateSystem launches the GB300 cylinder step on the legacy default
// stream, ordered with the reference's synchronous copies.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#pragma GCC visibility push(default)
#include "../../include/dsim2_abi.h"
#pragma GCC visibility pop
#include "common.cuh"
#include "engine.h"

namespace dsim {
static thread_local std::string g_last_error;
void set_last_error(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = std::string("dsim2 error ") + std::to_string(code) + ": " + buf;
}
void set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line) {
    set_last_error(kErrCuda, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
}
const char* last_error_message() { return g_last_error.c_str(); }
}  // namespace dsim

using namespace dsim;

namespace {
// The fine filter grid of the last grid arrays seen, with the device content
// hashes of the arrays it was built from to detect a change.
struct FineCache {
    bool valid = false;
    uint32_t n = 0, maxFPC = 0, nF = 0, k = 0;
    float L = 0.0f;
    const void* ptrs[3] = {nullptr, nullptr, nullptr};  // fibers, cube counts, cube lists
    uint64_t hash[3] = {0, 0, 0};                        // their contents when built
    unsigned long long* hashDev = nullptr;               // 3 device words (kept across releases)
    uint32_t* start = nullptr;
    float4* rec = nullptr;
    uint32_t* pos = nullptr;
    void release() {
        cudaFree(start); cudaFree(rec); cudaFree(pos);
        start = nullptr; rec = nullptr; pos = nullptr;
        valid = false;
    }
};
struct State {
    std::mutex mu;
    FineCache fine;
    int fineMode = -1;
    int last_status = 0;
    const float4* fibers = nullptr;
    uint32_t nF = 0;
    const uint32_t* boundList = nullptr;
    const float4* replay = nullptr;
    uint32_t* counts = nullptr;
    uint32_t* status = nullptr;
};
State& S() {
    static State s;
    return s;
}
void fail(int code) { S().last_status = code; }

// Points g at the fine filter grid of its arrays; false leaves g on the full
// list scan.  Each call hashes the three arrays on the device (one read each,
// nothing copied back); only when a pointer, a size or a hash differs from
// the cached grid's are the arrays copied to the host and the lists rebuilt.
bool fine_grid(State& s, CylDev& g) {
    if (s.fineMode == 0 || s.fineMode == 1) return false;
    FineCache& c = s.fine;
    const size_t ncell = (size_t)g.n * g.n * g.n;
    if (!c.hashDev && cudaMalloc(&c.hashDev, 3 * sizeof(unsigned long long)) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    const void* ptrs[3] = {g.fibers, g.cube_count, g.cubes};
    const size_t nw[3] = {(size_t)g.nF * 4, ncell, ncell * g.maxFPC};
    uint64_t h[3] = {0, 0, 0};
    if (hash_device_arrays(ptrs, nw, 3, c.hashDev, h, 0) != kOk) {
        cudaGetLastError();
        return false;
    }
    const bool same = c.valid && c.n == g.n && c.maxFPC == g.maxFPC && c.nF == g.nF && memcmp(&c.L, &g.L, 4) == 0 &&
                      memcmp(c.ptrs, ptrs, sizeof(ptrs)) == 0 && memcmp(c.hash, h, sizeof(h)) == 0;
    if (!same) {
        c.release();
        std::vector<float> fib((size_t)g.nF * 4);
        std::vector<uint32_t> cc(ncell), cubes(ncell * g.maxFPC);
        if ((!fib.empty() && cudaMemcpy(fib.data(), g.fibers, fib.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess) ||
            cudaMemcpy(cc.data(), g.cube_count, cc.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
            (!cubes.empty() && cudaMemcpy(cubes.data(), g.cubes, cubes.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess)) {
            cudaGetLastError();
            return false;
        }
        uint32_t k = 0;
        if (s.fineMode >= 2) {
            k = (uint32_t)s.fineMode;
        } else {
            double maxR = 0.0;
            for (uint32_t i = 0; i < g.nF; i++) {
                const double w = fib[4 * (size_t)i + 3];
                if (w > 0.0 && std::isfinite(w)) maxR = std::max(maxR, std::sqrt(w));
            }
            k = cyl_fine_size(g.n, g.L, maxR);
        }
        if (k < 2 || (uint64_t)(g.n * k) * (g.n * k) * (g.n * k) > (1ull << 24)) return false;
        std::vector<uint32_t> start, pos;
        std::vector<float> rec;
        // a grid the lists cannot describe (an index >= nF, a count above
        // maxFibersPerCube) keeps the full scan and its status bits
        if (cyl_fine_lists(fib.data(), g.nF, g.n, g.maxFPC, g.L, cc.data(), cubes.data(), k, start, pos, rec))
            return false;
        const size_t ne = std::max<size_t>(1, pos.size());
        if (cudaMalloc(&c.start, start.size() * 4) != cudaSuccess || cudaMalloc(&c.rec, ne * 16) != cudaSuccess ||
            cudaMalloc(&c.pos, ne * 4) != cudaSuccess ||
            cudaMemcpy(c.start, start.data(), start.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
            (!pos.empty() && (cudaMemcpy(c.rec, rec.data(), rec.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
                              cudaMemcpy(c.pos, pos.data(), pos.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess))) {
            cudaGetLastError();
            c.release();
            return false;
        }
        c.k = k; c.n = g.n; c.maxFPC = g.maxFPC; c.nF = g.nF; c.L = g.L;
        memcpy(c.ptrs, ptrs, sizeof(ptrs));
        memcpy(c.hash, h, sizeof(h));
        c.valid = true;
    }
    g.fine_start = c.start; g.fine_rec = c.rec; g.fine_pos = c.pos;
    g.fineK = c.k;
    g.fineInv = (float)c.k / g.L;
    return true;
}
}  // namespace

extern "C" {

void checkCUDA(void) {}

void allocateArray(void** devPtr, int size) {
    if (!devPtr || size < 0) { set_last_error(kErrInvalid, "allocateArray: bad argument"); fail(kErrInvalid); return; }
    cudaError_t e = cudaMalloc(devPtr, size > 0 ? (size_t)size : 1);
    if (e != cudaSuccess) {
        *devPtr = nullptr;
        cudaGetLastError();
        set_last_error(kErrNoMem, "allocateArray(%d): %s", size, cudaGetErrorString(e));
        fail(kErrNoMem);
    }
}

void freeArray(void* devPtr) {
    if (devPtr) cudaFree(devPtr);
}

void threadSync(void) {
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) { set_last_cuda_error(e, "threadSync", __FILE__, __LINE__); fail(kErrCuda); }
}

void copyArrayFromDevice(void* host, const void* device, unsigned int vbo, int size) {
    if (vbo) { set_last_error(kErrInvalid, "copyArrayFromDevice: OpenGL buffers are unavailable"); fail(kErrInvalid); return; }
    if (size <= 0) return;
    cudaError_t e = cudaMemcpy(host, device, (size_t)size, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) { set_last_cuda_error(e, "copyArrayFromDevice", __FILE__, __LINE__); fail(kErrCuda); }
}

void copyArrayToDevice(void* device, const void* host, int offset, int size) {
    if (size <= 0) return;
    cudaError_t e = cudaMemcpy((char*)device + offset, host, (size_t)size, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { set_last_cuda_error(e, "copyArrayToDevice", __FILE__, __LINE__); fail(kErrCuda); }
}

void registerGLBufferObject(unsigned int) {
    set_last_error(kErrInvalid, "registerGLBufferObject: OpenGL interop is unavailable");
    fail(kErrInvalid);
}
void unregisterGLBufferObject(unsigned int) {
    set_last_error(kErrInvalid, "unregisterGLBufferObject: OpenGL interop is unavailable");
    fail(kErrInvalid);
}

void bindFiberList(float* ptr, int size) {
    std::lock_guard<std::mutex> lk(S().mu);
    S().fibers = reinterpret_cast<const float4*>(ptr);
    S().nF = size > 0 ? (uint32_t)size : 0u;
}
void unbindFiberList(void) { std::lock_guard<std::mutex> lk(S().mu); S().fibers = nullptr; S().nF = 0; }
void bindCubeList(unsigned int* ptr, int) { std::lock_guard<std::mutex> lk(S().mu); S().boundList = ptr; }
void unbindCubeList(void) { std::lock_guard<std::mutex> lk(S().mu); S().boundList = nullptr; }

void integrateSystem(float* pos, unsigned int* randSeed, float deltaTime, float* fiberPos,
                     float permeability, float intraAdc, float extraAdc, float myelinAdc,
                     int numBodies, dsim_float3 gradient, float phaseConstant,
                     unsigned int* cubeCounters, unsigned int* cubeList, float cubeLength,
                     unsigned int numCubes, unsigned int maxFibersPerCube, float myelinRadius,
                     unsigned int iterations) {
    State& s = S();
    std::lock_guard<std::mutex> lk(s.mu);
    if (numBodies <= 0 || iterations == 0) return;
    if (!pos || !randSeed || !cubeCounters || (!cubeList && !s.boundList) || numCubes == 0) {
        set_last_error(kErrInvalid, "integrateSystem: null array or empty grid");
        fail(kErrInvalid);
        return;
    }
    if (!s.status) {
        if (cudaMalloc(&s.status, 4) != cudaSuccess || cudaMemset(s.status, 0, 4) != cudaSuccess) {
            set_last_error(kErrCuda, "integrateSystem: status word");
            fail(kErrCuda);
            return;
        }
    }
    CylDev g;
    g.cube_fibers = nullptr;  // the reference's own grid arrays: fiber indices only
    g.fine_start = nullptr; g.fine_rec = nullptr; g.fine_pos = nullptr;
    g.fineK = 0; g.fineInv = 0.0f;
    g.fibers = fiberPos ? reinterpret_cast<const float4*>(fiberPos) : s.fibers;
    g.cube_count = cubeCounters;
    g.cubes = cubeList ? cubeList : s.boundList;
    g.n = numCubes;
    g.maxFPC = maxFibersPerCube;
    g.L = cubeLength;
    g.nF = s.nF;
    if (!g.fibers || g.nF == 0) {
        set_last_error(kErrInvalid, "integrateSystem: bindFiberList(fibers, count) must precede the step");
        fail(kErrInvalid);
        return;
    }
    fine_grid(s, g);
    CylStepArgs a;
    memset(&a, 0, sizeof(a));
    // integrateSystem, dSim2/src/spinSystem.cu:148-153: sd = sqrt(2 ADC dt)
    a.intraSd = sqrtf(2.0f * intraAdc * deltaTime);
    a.extraSd = sqrtf(2.0f * extraAdc * deltaTime);
    a.myelinSd = sqrtf(2.0f * myelinAdc * deltaTime);
    a.T2fiber = a.T2myelin = a.T2outside = INFINITY;
    a.perm = permeability;
    a.inRadPropSq = myelinRadius * myelinRadius;
    a.clampHi = 1.0f - 0.005f;
    a.clampLo = -1.0f + 0.005f;
    a.dt = deltaTime;
    a.pc = phaseConstant;
    a.gx = gradient.x; a.gy = gradient.y; a.gz = gradient.z;
    a.iterations = iterations;
    a.draws = s.replay;
    a.status = s.status;
    a.counts = s.counts;
    CylSpinsDev sp;
    sp.pos = reinterpret_cast<float4*>(pos);
    sp.seed4 = randSeed;
    sp.mag = nullptr;
    sp.N = (uint32_t)numBodies;
    int rc = launch_cyl_step(g, a, sp, s.replay ? kRngReplay : kRngPhiloxPerSpinKey, 0);
    if (rc) fail(rc);
}

void integrateSystemVbo(unsigned int, unsigned int*, float, float*, float, float, float, float, int,
                        dsim_float3, float, unsigned int*, unsigned int*, float, unsigned int,
                        unsigned int, float, unsigned int) {
    set_last_error(kErrInvalid, "integrateSystemVbo: OpenGL position buffers are unavailable");
    fail(kErrInvalid);
}

const char* dsim2_last_error(void) { return last_error_message(); }
int dsim2_last_status(void) {
    int v = S().last_status;
    S().last_status = 0;
    return v;
}
void dsim2_set_replay(const float* draws, unsigned int* counts) {
    std::lock_guard<std::mutex> lk(S().mu);
    S().replay = reinterpret_cast<const float4*>(draws);
    S().counts = counts;
}
void dsim2_set_fine(int k) {
    std::lock_guard<std::mutex> lk(S().mu);
    S().fineMode = k;
    S().fine.release();
}
unsigned int dsim2_status(void) {
    State& s = S();
    std::lock_guard<std::mutex> lk(s.mu);
    if (!s.status) return 0;
    uint32_t v = 0;
    cudaMemcpy(&v, s.status, 4, cudaMemcpyDeviceToHost);
    cudaMemset(s.status, 0, 4);
    return v;
}

}  // extern "C"
