/*
 * dsim3_abi.h -- drop-in replacement for the dSim3 plugin boundary
 * (rfdougherty/dSim dSim3/src/spinSystem.cuh:1-59), exported by libdsim3.so.
 *
 * The reference's host code (SpinSystem in dSim3/src/spinSystem.cpp) calls
 * only these functions to reach the GPU; linking it against libdsim3.so
 * instead of the reference's spinSystem.cu runs the same simulation on a
 * GB300.  Signatures are the reference's; every function keeps its void
 * return (as the reference) and records failures for dsim_last_error().
 *
 * Types: the reference passes its own float3 {x,y,z} by value and its
 * 12-byte spinData {float signalMagnitude; float signalPhase;
 * uint8 compartmentType; uint16 insideFiber;} records by pointer.
 */
#ifndef DSIM3_ABI_H
#define DSIM3_ABI_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#ifndef DSIM_ABI_TYPES_DEFINED
#define DSIM_ABI_TYPES_DEFINED
typedef struct { float x, y, z; } dsim_float3;
#endif
/* spinData, dSim3/src/dSimDataTypes.h:9-24 (12 bytes with padding) */
typedef struct {
    float signalMagnitude;
    float signalPhase;
    uint8_t compartmentType;
    uint16_t insideFiber;
} dsim_spinData;

/* spinSystem.cuh:4 -- no-op (device 0 is used; kept for link compatibility) */
void checkCUDA(void);
/* spinSystem.cuh:6-7 -- cudaMalloc / cudaFree of caller-owned device arrays */
void allocateArray(void** devPtr, int size);
void freeArray(void* devPtr);
/* spinSystem.cuh:9 -- block until all queued work has finished */
void threadSync(void);
/* spinSystem.cuh:11-12 -- synchronous copies.  vbo != 0 (OpenGL buffer) is
 * unavailable on this build and records DSIM_EINVAL. */
void copyArrayFromDevice(void* host, const void* device, unsigned int vbo, int size);
void copyArrayToDevice(void* device, const void* host, int offset, int size);
/* spinSystem.cuh:13-14 -- OpenGL interop: unavailable (records an error) */
void registerGLBufferObject(unsigned int vbo);
void unregisterGLBufferObject(unsigned int vbo);
/* spinSystem.cuh:15 -- set a simulation constant by the reference's
 * __constant__ symbol name (k_reflectionType, k_triSearchMethod, k_nFibers,
 * k_nCompartments, k_permeability, k_deltaTime, k_T2Values, k_stdDevs,
 * k_numCubes, k_totalNumCubes, k_maxTrianglesPerCube, k_cubeLength).  For
 * k_T2Values and k_stdDevs the reference passes the address of a device
 * pointer variable (spinSystem.cpp:273-277); the full pointer is read and
 * the four per-compartment values are fetched from the device. */
void copyConstantToDevice(void* device, const void* host, int offset, int size);
/* spinSystem.cuh:17-32 -- record the substrate arrays (sizes in elements) */
void bindCubeCounter(unsigned int* ptr, int size);
void unbindCubeCounter(void);
void bindTrianglesInCubes(unsigned int* ptr, int size);
void unbindTrianglesInCubes(void);
void bindVertices(float* ptr, int size);
void unbindVertices(void);
void bindTriangleHelpers(float* ptr, int size);
void unbindTriangleHelpers(void);
void bindRTreeArray(float* ptr, int size);
void unbindRTreeArray(void);
void bindTreeIndexArray(unsigned int* ptr, int size);
void unbindTreeIndexArray(void);
void bindTriInfo(unsigned int* ptr, int size);
void unbindTriInfo(void);
/* spinSystem.cuh:34-45 -- advance numBodies spins `iterations` steps.
 * pos: float3[N] positions, randSeed: uint2[N] (used as per-spin Philox
 * keys, advanced on return), spinInfo: spinData[N]; all updated in place.
 * trianglesInCubes / cubeCounter: the dense grid from populateCubes
 * (spinSystem.cpp:1094-1352), converted once to compact cell lists. */
void integrateSystem(float* pos, unsigned int* randSeed, dsim_spinData* spinInfo, float deltaTime,
                     float permeability, int numBodies, dsim_float3 magneticGradient,
                     float phaseConstant, unsigned int iterations, unsigned int* trianglesInCubes,
                     unsigned int* cubeCounter);
/* spinSystem.cuh:47-58 -- OpenGL position buffer: unavailable (records an error) */
void integrateSystemVBO(unsigned int vboPos, unsigned int* randSeed, dsim_spinData* spinInfo,
                        float deltaTime, float permeability, int numBodies,
                        dsim_float3 magneticGradient, float phaseConstant, unsigned int iterations,
                        unsigned int* trianglesInCubes, unsigned int* cubeCounter);

/* ---- additions (no counterpart in the reference) ------------------------ */
/* last failure message and code of the calls above (0 when none) */
const char* dsim3_last_error(void);
int dsim3_last_status(void);
/* Replay: when draws is a device array of iterations*numBodies float4
 * (n.x, n.y, n.z, u), the next integrateSystem calls take their steps from
 * it instead of Philox (NULL restores Philox).  counts, when non-NULL, is a
 * device uint32[2N] accumulator of {reflections, permeations}. */
void dsim3_set_replay(const float* draws, unsigned int* counts);
/* OR of the kernels' status bits since the last call (cleared on read) */
unsigned int dsim3_status(void);

#ifdef __cplusplus
}
#endif
#endif
