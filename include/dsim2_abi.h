/*
 * dsim2_abi.h -- drop-in replacement for the dSim2 (cylinder) plugin boundary
 * (rfdougherty/dSim dSim2/src/spinSystem.cuh:1-62), exported by libdsim2.so.
 *
 * Same signatures as the reference.  State layout is the reference's GPU
 * layout: pos = float4[N] {x, y, z, phase}; randSeed = uint4[N] {s0, s1, z, w}
 * where w is the index of the fiber containing the spin (UINT_MAX outside),
 * as in dSim2/src/spinKernel.cu:256-265.  This build also keeps the
 * three-compartment state of the reference's CPU step in z (0 = derive from
 * w, otherwise 1 + {0 core, 1 myelin, 2 outside}) and steps with the CPU
 * path's membrane semantics (dSim2/src/spinKernelCpu.cpp:312-641); the ABI
 * carries no magnitude, so T2 decay is not applied on this boundary.
 */
#ifndef DSIM2_ABI_H
#define DSIM2_ABI_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#ifndef DSIM_ABI_TYPES_DEFINED
#define DSIM_ABI_TYPES_DEFINED
typedef struct { float x, y, z; } dsim_float3;
#endif

/* spinSystem.cuh:4-14: device management and synchronous copies */
void checkCUDA(void);
void allocateArray(void** devPtr, int size);
void freeArray(void* devPtr);
void threadSync(void);
void copyArrayFromDevice(void* host, const void* device, unsigned int vbo, int size);
void copyArrayToDevice(void* device, const void* host, int offset, int size);
void registerGLBufferObject(unsigned int vbo);   /* unavailable: records an error */
void unregisterGLBufferObject(unsigned int vbo); /* unavailable: records an error */
/* spinSystem.cuh:16-19: fibers float4[size] {x, y, z, r^2}; cell list uint[size] */
void bindFiberList(float* ptr, int size);
void unbindFiberList(void);
void bindCubeList(unsigned int* ptr, int size);
void unbindCubeList(void);
/* spinSystem.cuh:21-40: intraAdc/extraAdc/myelinAdc are already divided by
 * spaceScale^2; myelinRadius is the inner-radius proportion; cubeCounters /
 * cubeList are the dense grid of addEntities (dSim2/src/spinSystem.cpp:483-745). */
void integrateSystem(float* pos, unsigned int* randSeed, float deltaTime, float* fiberPos,
                     float permeability, float intraAdc, float extraAdc, float myelinAdc,
                     int numBodies, dsim_float3 magneticGradient, float phaseConstant,
                     unsigned int* cubeCounters, unsigned int* cubeList, float cubeLength,
                     unsigned int numCubes, unsigned int maxFibersPerCube, float myelinRadius,
                     unsigned int iterations);
/* spinSystem.cuh:42-61: OpenGL position buffer: unavailable (records an error) */
void integrateSystemVbo(unsigned int vboPos, unsigned int* randSeed, float deltaTime,
                        float* fiberPos, float permeability, float intraAdc, float extraAdc,
                        float myelinAdc, int numBodies, dsim_float3 magneticGradient,
                        float phaseConstant, unsigned int* cubeCounters, unsigned int* cubeList,
                        float cubeLength, unsigned int numCubes, unsigned int maxFibersPerCube,
                        float myelinRadius, unsigned int iterations);

/* ---- additions (no counterpart in the reference) ------------------------ */
const char* dsim2_last_error(void);
int dsim2_last_status(void);
/* replay draws (device float4[iterations*N]) and collision counters
 * (device uint32[2N]); NULL restores Philox / disables counting */
void dsim2_set_replay(const float* draws, unsigned int* counts);
unsigned int dsim2_status(void);
/* Fine filter grid over the caller's grid arrays: integrateSystem copies the
 * fibers, cubeCounters and cubeList back each call, rebuilds the fine lists
 * when their contents changed, and then tests a spin outside every fiber
 * against its fine cell's entries only, with results equal to the full list
 * scan.  k < 0: the default size (initially); 0 or 1: full list scan;
 * k >= 2: k fine cells per grid-cell edge. */
void dsim2_set_fine(int k);

#ifdef __cplusplus
}
#endif
#endif
