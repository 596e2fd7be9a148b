// cyl_common.cuh -- the dSim2 membrane rules for one step of one spin, shared
// by the cylinder step kernel (cyl.cu) and the multi-job batch kernel.
//
// Reference (rfdougherty/dSim): cpuIntegrate dSim2/src/spinKernelCpu.cpp:312-641,
// distToCenterSq :71-82, calcCubePos/calcCubeHash dSim2/src/spinSystem.cpp:413-433.
#pragma once
#include "common.cuh"
#include "engine.h"

namespace dsim {

// calcCubeHash(calcCubePos(p)): the float3 division of the reference's header
// multiplies by the reciprocal; clamping happens in the hash.
__device__ __forceinline__ uint32_t cyl_cell(float px, float py, float pz, float L, uint32_t n) {
    float inv = 1.0f / L;
    float cx = floorf((px + 1.0f) * inv);
    float cy = floorf((py + 1.0f) * inv);
    float cz = floorf((pz + 1.0f) * inv);
    float hi = (float)(n - 1);
    cx = fmaxf(fminf(cx, hi), 0.0f);
    cy = fmaxf(fminf(cy, hi), 0.0f);
    cz = fmaxf(fminf(cz, hi), 0.0f);
    return (uint32_t)((int)((float)(n * n) * cz) + (int)((float)n * cy) + (int)cx);
}

__device__ __forceinline__ float cyl_dist_sq(float px, float py, float pz, float4 f) {
    if (f.x == 2.0f) return (pz - f.z) * (pz - f.z) + (py - f.y) * (py - f.y);
    else if (f.z == 2.0f) return (px - f.x) * (px - f.x) + (py - f.y) * (py - f.y);
    return (px - f.x) * (px - f.x) + (pz - f.z) * (pz - f.z);
}

// Membrane test of the proposed position p (from o) for a spin in region imo
// (0 core, 1 myelin, 2 outside) with nearest fiber `nearest`: a rejected step
// puts p back to o; permeation and the end-position region update imo.
__device__ __forceinline__ void cyl_membranes(const CylDev& g, float ox, float oy, float oz,
                                              float& px, float& py, float& pz, float u, float perm,
                                              float inR, uint32_t& imo, uint32_t& nearest,
                                              uint32_t& nrej, uint32_t& nperm, uint32_t& status) {
    if (perm < 1.0f) {
        if (imo < 2) {
            float4 f = __ldg(g.fibers + nearest);
            float radSq = f.w;
            float cur = cyl_dist_sq(px, py, pz, f);
            if (imo == 0) {
                if ((cur > inR * radSq) & (cur <= radSq)) {
                    if (u >= perm) { px = ox; py = oy; pz = oz; nrej++; }
                    else { imo = 1; nperm++; }
                } else if (cur > radSq) {
                    if (u < 1.0f - perm) { px = ox; py = oy; pz = oz; nrej++; }
                    else if ((1.0f - perm < u) & (u < 1.0f - perm * perm)) {
                        px = ox; py = oy; pz = oz; imo = 1; nrej++;
                    } else { imo = 2; nperm++; }
                }
            } else {
                if (cur > radSq) {
                    if (u >= perm) { px = ox; py = oy; pz = oz; nrej++; }
                    else { imo = 2; nperm++; }
                } else if (cur < inR * radSq) {
                    if (u >= perm) { px = ox; py = oy; pz = oz; nrej++; }
                    else { imo = 0; nperm++; }
                }
            }
            float endD = cyl_dist_sq(px, py, pz, f);
            if (endD > radSq) imo = 2;
            else if (endD < inR * radSq) imo = 0;
            else imo = 1;
        } else {
            // a cell's entries: the inline record when the grid has them (the
            // index is read only when the spin changes region), else the index
            // and then the fiber
            uint32_t cube = cyl_cell(px, py, pz, g.L, g.n);
            uint32_t cnt = __ldg(g.cube_count + cube);
            const uint32_t* list = g.cubes + (size_t)cube * g.maxFPC;
            const float4* inl = g.cube_fibers ? g.cube_fibers + (size_t)cube * g.maxFPC : nullptr;
            for (uint32_t j = 0; j < cnt; j++) {
                float4 f;
                uint32_t fi = 0;
                if (inl) {
                    f = __ldg(inl + j);
                } else {
                    fi = __ldg(list + j);
                    if (fi >= g.nF) { status |= kStatusBadCell; continue; }
                    f = __ldg(g.fibers + fi);
                }
                float radSq = f.w;
                float cur = cyl_dist_sq(px, py, pz, f);
                if ((cur <= radSq) & (cur > inR * radSq)) {
                    if (u >= perm) { px = ox; py = oy; pz = oz; nrej++; }
                    else { imo = 1; nearest = inl ? __ldg(list + j) : fi; nperm++; }
                } else if (cur < inR * radSq) {
                    if (u < 1.0f - perm) { px = ox; py = oy; pz = oz; nrej++; }
                    else if ((1.0f - perm < u) & (u < 1.0f - perm * perm)) {
                        px = ox; py = oy; pz = oz; nearest = inl ? __ldg(list + j) : fi; imo = 1; nrej++;
                    } else { imo = 0; nearest = inl ? __ldg(list + j) : fi; nperm++; }
                }
            }
            if (imo == 2) {
                cube = cyl_cell(px, py, pz, g.L, g.n);
                cnt = __ldg(g.cube_count + cube);
                list = g.cubes + (size_t)cube * g.maxFPC;
                inl = g.cube_fibers ? g.cube_fibers + (size_t)cube * g.maxFPC : nullptr;
                for (uint32_t j = 0; j < cnt; j++) {
                    float4 f;
                    if (inl) {
                        f = __ldg(inl + j);
                    } else {
                        const uint32_t fi = __ldg(list + j);
                        if (fi >= g.nF) { status |= kStatusBadCell; continue; }
                        f = __ldg(g.fibers + fi);
                    }
                    float nd = cyl_dist_sq(px, py, pz, f);
                    if (nd < inR * f.w) { px = ox; py = oy; pz = oz; nrej++; }
                    else if (nd < f.w) { px = ox; py = oy; pz = oz; nrej++; }
                }
            }
        }
    }
}

}  // namespace dsim
