/* host_abi.cpp -- host-memory implementation of the reference's C-ABI
 * (dSim3/src/spinSystem.cuh, dSim2/src/spinSystem.cuh) so that the
 * reference's CPU path runs with "device" arrays in host memory.  Test
 * infrastructure for oracle/_ref/ only.  The GPU entry points
 * (integrateSystem*) abort: the harnesses run the reference's CPU path. */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include "spinSystem.h"
#include "spinSystem.cuh"

extern "C" {
void checkCUDA() {}
void allocateArray(void** devPtr, int size) { *devPtr = calloc(1, size > 0 ? (size_t)size : 1); }
void freeArray(void*) {}
void threadSync() {}
void copyArrayFromDevice(void* host, const void* device, unsigned int, int size) {
    if (size > 0 && host != device) memcpy(host, device, (size_t)size);
}
void copyArrayToDevice(void* device, const void* host, int offset, int size) {
    if (size > 0) memcpy((char*)device + offset, host, (size_t)size);
}
#ifdef DSIM2_ABI
void bindFiberList(float*, int) {}
void unbindFiberList() {}
void bindCubeList(uint*, int) {}
void unbindCubeList() {}
void integrateSystem(float*, uint*, float, float*, float, float, float, float, int, float3, float,
                     uint*, uint*, float, uint, uint, float, uint) {
    fprintf(stderr, "harness: GPU path not available in the reference harness\n");
    abort();
}
void integrateSystemVbo(uint, uint*, float, float*, float, float, float, float, int, float3, float,
                        uint*, uint*, float, uint, uint, float, uint) {
    fprintf(stderr, "harness: GPU path not available in the reference harness\n");
    abort();
}
#else
void copyConstantToDevice(void*, const void*, int, int) {}
void bindCubeCounter(uint*, int) {}
void unbindCubeCounter() {}
void bindTrianglesInCubes(uint*, int) {}
void unbindTrianglesInCubes() {}
void bindVertices(float*, int) {}
void unbindVertices() {}
void bindTriangleHelpers(float*, int) {}
void unbindTriangleHelpers() {}
void bindRTreeArray(float*, int) {}
void unbindRTreeArray() {}
void bindTreeIndexArray(uint*, int) {}
void unbindTreeIndexArray() {}
void bindTriInfo(uint*, int) {}
void unbindTriInfo() {}
void integrateSystem(float*, uint*, spinData*, float, float, int, float3, float, uint, uint*, uint*) {
    fprintf(stderr, "harness: GPU path not available in the reference harness\n");
    abort();
}
void integrateSystemVBO(uint, uint*, spinData*, float, float, int, float3, float, uint, uint*, uint*) {
    fprintf(stderr, "harness: GPU path not available in the reference harness\n");
    abort();
}
#endif
}
