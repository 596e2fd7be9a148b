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
    float cx = floor_small((px + 1.0f) * inv);
    float cy = floor_small((py + 1.0f) * inv);
    float cz = floor_small((pz + 1.0f) * inv);
    float hi = (float)(n - 1);
    cx = fmaxf(fminf(cx, hi), 0.0f);
    cy = fmaxf(fminf(cy, hi), 0.0f);
    cz = fmaxf(fminf(cz, hi), 0.0f);
    // the reference's float products (float)(n*n) * cz etc. are exact integers
    // while n^3 < 2^24 (its grid has at most 100 cells per axis), so integer
    // arithmetic gives the same index
    return n * n * uint_small(cz) + n * uint_small(cy) + uint_small(cx);
}

__device__ __forceinline__ float cyl_dist_sq(float px, float py, float pz, float4 f) {
    if (f.x == 2.0f) return (pz - f.z) * (pz - f.z) + (py - f.y) * (py - f.y);
    else if (f.z == 2.0f) return (px - f.x) * (px - f.x) + (py - f.y) * (py - f.y);
    return (px - f.x) * (px - f.x) + (pz - f.z) * (pz - f.z);
}

// The spin's fine cell inside its grid cell `cube` (the grid's own cell of
// the point): the fine coordinate, clamped to the grid cell's fineK cells.
__device__ __forceinline__ uint32_t cyl_fine_cell(const CylDev& g, float px, float py, float pz, uint32_t cube) {
    const uint32_t n = g.n, k = g.fineK, nk = n * k;
    const uint32_t cx = cube % n, cy = (cube / n) % n, cz = cube / (n * n);
    const float hi = (float)(k - 1);
    const float sx = fminf(fmaxf(floor_small((px + 1.0f) * g.fineInv) - (float)(cx * k), 0.0f), hi);
    const float sy = fminf(fmaxf(floor_small((py + 1.0f) * g.fineInv) - (float)(cy * k), 0.0f), hi);
    const float sz = fminf(fmaxf(floor_small((pz + 1.0f) * g.fineInv) - (float)(cz * k), 0.0f), hi);
    return ((cz * k + uint_small(sz)) * nk + (cy * k + uint_small(sy))) * nk + cx * k + uint_small(sx);
}

// One list entry (fiber record f, list position j) of the first pass of a
// spin outside every fiber, tested at the current p.
__device__ __forceinline__ void cyl_outside_entry(float4 f, const uint32_t* list, uint32_t j, float ox, float oy,
                                                  float oz, float& px, float& py, float& pz, float u, float perm,
                                                  float inR, uint32_t& imo, uint32_t& nearest, uint32_t& nrej,
                                                  uint32_t& nperm, bool& moved, bool& inside) {
    float radSq = f.w;
    float cur = cyl_dist_sq(px, py, pz, f);
    inside |= (cur < inR * radSq) | (cur < radSq);
    if ((cur <= radSq) & (cur > inR * radSq)) {
        if (u >= perm) { px = ox; py = oy; pz = oz; nrej++; moved = true; }
        else { imo = 1; nearest = __ldg(list + j); nperm++; }
    } else if (cur < inR * radSq) {
        if (u < 1.0f - perm) { px = ox; py = oy; pz = oz; nrej++; moved = true; }
        else if ((1.0f - perm < u) & (u < 1.0f - perm * perm)) {
            px = ox; py = oy; pz = oz; nearest = __ldg(list + j); imo = 1; nrej++;
            moved = true;
        } else { imo = 0; nearest = __ldg(list + j); nperm++; }
    }
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
            // The second pass below rejects the step once for each fiber of
            // the end position's cell with d^2 < inR r^2 or d^2 < r^2.  While
            // this pass moves nothing, the end position is the one tested
            // here, so `inside` (that test on every entry) decides whether
            // the second pass can change anything; if not, it is skipped.
            bool moved = false, inside = false;
            const bool fine = g.fine_start != nullptr && inR <= 1.0f;
            uint32_t j = 0;
            if (fine) {
                // While the tested point is p, only the fine cell's entries
                // can act; after the first rejection (p = o) the rest of the
                // list is tested at o entry by entry.
                const uint32_t fc = cyl_fine_cell(g, px, py, pz, cube);
                const uint32_t e1 = __ldg(g.fine_start + fc + 1);
                j = cnt;
                uint32_t jm = 0;
                for (uint32_t e = __ldg(g.fine_start + fc); e < e1; e++) {
                    const uint32_t jj = __ldg(g.fine_pos + e);
                    cyl_outside_entry(__ldg(g.fine_rec + e), list, jj, ox, oy, oz, px, py, pz, u, perm, inR, imo,
                                      nearest, nrej, nperm, moved, inside);
                    if (moved) { jm = jj; break; }
                }
                // the entries after position jm, at o: when o lies in the same
                // grid cell, o's fine cell holds every one that can act there
                if (moved) {
                    if (cyl_cell(px, py, pz, g.L, g.n) == cube) {
                        const uint32_t fo = cyl_fine_cell(g, px, py, pz, cube);
                        const uint32_t eo1 = __ldg(g.fine_start + fo + 1);
                        for (uint32_t e = __ldg(g.fine_start + fo); e < eo1; e++) {
                            const uint32_t jj = __ldg(g.fine_pos + e);
                            if (jj <= jm) continue;
                            cyl_outside_entry(__ldg(g.fine_rec + e), list, jj, ox, oy, oz, px, py, pz, u, perm, inR,
                                              imo, nearest, nrej, nperm, moved, inside);
                        }
                    } else {
                        j = jm + 1;
                    }
                }
            }
            for (; j < cnt; j++) {
                float4 f;
                if (inl) {
                    f = __ldg(inl + j);
                } else {
                    const uint32_t fi = __ldg(list + j);
                    if (fi >= g.nF) { status |= kStatusBadCell; continue; }
                    f = __ldg(g.fibers + fi);
                }
                cyl_outside_entry(f, list, j, ox, oy, oz, px, py, pz, u, perm, inR, imo, nearest, nrej, nperm,
                                  moved, inside);
            }
            if (imo == 2 && (moved || inside)) {
                cube = cyl_cell(px, py, pz, g.L, g.n);
                cnt = __ldg(g.cube_count + cube);
                list = g.cubes + (size_t)cube * g.maxFPC;
                inl = g.cube_fibers ? g.cube_fibers + (size_t)cube * g.maxFPC : nullptr;
                if (fine && moved) {
                    // p = o for the whole pass, so o's fine cell stands for the list
                    const uint32_t fc = cyl_fine_cell(g, px, py, pz, cube);
                    const uint32_t e1 = __ldg(g.fine_start + fc + 1);
                    for (uint32_t e = __ldg(g.fine_start + fc); e < e1; e++) {
                        const float4 f = __ldg(g.fine_rec + e);
                        float nd = cyl_dist_sq(px, py, pz, f);
                        if (nd < inR * f.w) { px = ox; py = oy; pz = oz; nrej++; }
                        else if (nd < f.w) { px = ox; py = oy; pz = oz; nrej++; }
                    }
                } else {
                    for (uint32_t j2 = 0; j2 < cnt; j2++) {
                        float4 f;
                        if (inl) {
                            f = __ldg(inl + j2);
                        } else {
                            const uint32_t fi = __ldg(list + j2);
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
}

// ---- the same rules with positions and distances in double ----------------
// (the cylinder precision form, DSIM_JOB_PRECISE).  Parameters are the
// reference's float values (fiber records, r^2, inner radius proportion
// squared, permeability, draws) promoted to double; every position-dependent
// quantity is formed in double in the same order as the FP32 rules above.
__device__ __forceinline__ uint32_t cyl_cell64(double px, double py, double pz, float L, uint32_t n) {
    const double inv = 1.0 / (double)L;
    const double hi = (double)(n - 1);
    const double cx = fmax(fmin(floor((px + 1.0) * inv), hi), 0.0);
    const double cy = fmax(fmin(floor((py + 1.0) * inv), hi), 0.0);
    const double cz = fmax(fmin(floor((pz + 1.0) * inv), hi), 0.0);
    return (uint32_t)cz * n * n + (uint32_t)cy * n + (uint32_t)cx;
}

__device__ __forceinline__ double cyl_dist_sq64(double px, double py, double pz, float4 f) {
    const double fx = f.x, fy = f.y, fz = f.z;
    if (f.x == 2.0f) return (pz - fz) * (pz - fz) + (py - fy) * (py - fy);
    else if (f.z == 2.0f) return (px - fx) * (px - fx) + (py - fy) * (py - fy);
    return (px - fx) * (px - fx) + (pz - fz) * (pz - fz);
}

// the fine cell of p in grid cell `cube`; the fine lists are registered in
// double against cells widened by 1e-5, so every entry able to act at p is in
// the list of the cell this picks
__device__ __forceinline__ uint32_t cyl_fine_cell64(const CylDev& g, double px, double py, double pz, uint32_t cube) {
    const uint32_t n = g.n, k = g.fineK, nk = n * k;
    const uint32_t cx = cube % n, cy = (cube / n) % n, cz = cube / (n * n);
    const double hi = (double)(k - 1), inv = (double)g.fineInv;
    const double sx = fmin(fmax(floor((px + 1.0) * inv) - (double)(cx * k), 0.0), hi);
    const double sy = fmin(fmax(floor((py + 1.0) * inv) - (double)(cy * k), 0.0), hi);
    const double sz = fmin(fmax(floor((pz + 1.0) * inv) - (double)(cz * k), 0.0), hi);
    return ((cz * k + (uint32_t)sz) * nk + (cy * k + (uint32_t)sy)) * nk + cx * k + (uint32_t)sx;
}

__device__ __forceinline__ void cyl_outside_entry64(float4 f, const uint32_t* list, uint32_t j, double ox, double oy,
                                                    double oz, double& px, double& py, double& pz, double u,
                                                    double perm, double inR, uint32_t& imo, uint32_t& nearest,
                                                    uint32_t& nrej, uint32_t& nperm, bool& moved, bool& inside) {
    const double radSq = f.w;
    const double cur = cyl_dist_sq64(px, py, pz, f);
    inside |= (cur < inR * radSq) | (cur < radSq);
    if ((cur <= radSq) & (cur > inR * radSq)) {
        if (u >= perm) { px = ox; py = oy; pz = oz; nrej++; moved = true; }
        else { imo = 1; nearest = __ldg(list + j); nperm++; }
    } else if (cur < inR * radSq) {
        if (u < 1.0 - perm) { px = ox; py = oy; pz = oz; nrej++; moved = true; }
        else if ((1.0 - perm < u) & (u < 1.0 - perm * perm)) {
            px = ox; py = oy; pz = oz; nearest = __ldg(list + j); imo = 1; nrej++;
            moved = true;
        } else { imo = 0; nearest = __ldg(list + j); nperm++; }
    }
}

__device__ __forceinline__ void cyl_membranes64(const CylDev& g, double ox, double oy, double oz, double& px,
                                                double& py, double& pz, double u, double perm, double inR,
                                                uint32_t& imo, uint32_t& nearest, uint32_t& nrej, uint32_t& nperm,
                                                uint32_t& status) {
    if (!(perm < 1.0)) return;
    if (imo < 2) {
        const float4 f = __ldg(g.fibers + nearest);
        const double radSq = f.w;
        const double cur = cyl_dist_sq64(px, py, pz, f);
        if (imo == 0) {
            if ((cur > inR * radSq) & (cur <= radSq)) {
                if (u >= perm) { px = ox; py = oy; pz = oz; nrej++; }
                else { imo = 1; nperm++; }
            } else if (cur > radSq) {
                if (u < 1.0 - perm) { px = ox; py = oy; pz = oz; nrej++; }
                else if ((1.0 - perm < u) & (u < 1.0 - perm * perm)) {
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
        const double endD = cyl_dist_sq64(px, py, pz, f);
        if (endD > radSq) imo = 2;
        else if (endD < inR * radSq) imo = 0;
        else imo = 1;
        return;
    }
    uint32_t cube = cyl_cell64(px, py, pz, g.L, g.n);
    uint32_t cnt = __ldg(g.cube_count + cube);
    const uint32_t* list = g.cubes + (size_t)cube * g.maxFPC;
    const float4* inl = g.cube_fibers ? g.cube_fibers + (size_t)cube * g.maxFPC : nullptr;
    bool moved = false, inside = false;
    const bool fine = g.fine_start != nullptr && inR <= 1.0;
    uint32_t j = 0;
    if (fine) {
        const uint32_t fc = cyl_fine_cell64(g, px, py, pz, cube);
        const uint32_t e1 = __ldg(g.fine_start + fc + 1);
        j = cnt;
        uint32_t jm = 0;
        for (uint32_t e = __ldg(g.fine_start + fc); e < e1; e++) {
            const uint32_t jj = __ldg(g.fine_pos + e);
            cyl_outside_entry64(__ldg(g.fine_rec + e), list, jj, ox, oy, oz, px, py, pz, u, perm, inR, imo, nearest,
                                nrej, nperm, moved, inside);
            if (moved) { jm = jj; break; }
        }
        if (moved) {
            if (cyl_cell64(px, py, pz, g.L, g.n) == cube) {
                const uint32_t fo = cyl_fine_cell64(g, px, py, pz, cube);
                const uint32_t eo1 = __ldg(g.fine_start + fo + 1);
                for (uint32_t e = __ldg(g.fine_start + fo); e < eo1; e++) {
                    const uint32_t jj = __ldg(g.fine_pos + e);
                    if (jj <= jm) continue;
                    cyl_outside_entry64(__ldg(g.fine_rec + e), list, jj, ox, oy, oz, px, py, pz, u, perm, inR, imo,
                                        nearest, nrej, nperm, moved, inside);
                }
            } else {
                j = jm + 1;
            }
        }
    }
    for (; j < cnt; j++) {
        float4 f;
        if (inl) {
            f = __ldg(inl + j);
        } else {
            const uint32_t fi = __ldg(list + j);
            if (fi >= g.nF) { status |= kStatusBadCell; continue; }
            f = __ldg(g.fibers + fi);
        }
        cyl_outside_entry64(f, list, j, ox, oy, oz, px, py, pz, u, perm, inR, imo, nearest, nrej, nperm, moved,
                            inside);
    }
    if (imo == 2 && (moved || inside)) {
        cube = cyl_cell64(px, py, pz, g.L, g.n);
        cnt = __ldg(g.cube_count + cube);
        list = g.cubes + (size_t)cube * g.maxFPC;
        inl = g.cube_fibers ? g.cube_fibers + (size_t)cube * g.maxFPC : nullptr;
        if (fine && moved) {
            const uint32_t fc = cyl_fine_cell64(g, px, py, pz, cube);
            const uint32_t e1 = __ldg(g.fine_start + fc + 1);
            for (uint32_t e = __ldg(g.fine_start + fc); e < e1; e++) {
                const float4 f = __ldg(g.fine_rec + e);
                const double nd = cyl_dist_sq64(px, py, pz, f);
                if (nd < inR * (double)f.w) { px = ox; py = oy; pz = oz; nrej++; }
                else if (nd < (double)f.w) { px = ox; py = oy; pz = oz; nrej++; }
            }
        } else {
            for (uint32_t j2 = 0; j2 < cnt; j2++) {
                float4 f;
                if (inl) {
                    f = __ldg(inl + j2);
                } else {
                    const uint32_t fi = __ldg(list + j2);
                    if (fi >= g.nF) { status |= kStatusBadCell; continue; }
                    f = __ldg(g.fibers + fi);
                }
                const double nd = cyl_dist_sq64(px, py, pz, f);
                if (nd < inR * (double)f.w) { px = ox; py = oy; pz = oz; nrej++; }
                else if (nd < (double)f.w) { px = ox; py = oy; pz = oz; nrej++; }
            }
        }
    }
}

// ---- the cell-local FP32 form (DSIM_JOB_LOCAL cylinder jobs) ---------------
// A position is a lattice origin G (a multiple of 1/16, exact in float) plus an
// FP32 offset p.  The distance to a fiber's axis is formed in the local frame,
// ((G - f) + p) per axis, which rounds about 16x finer than the absolute FP32
// coordinates of the reference's step.  Each membrane decision compares d^2
// with inR r^2 and r^2; where the FP32 d^2 lies within its error band of
// either, the decision is taken from the FP64 distance at the exact position
// G + p, as the FP64 form would take it there.  Grid and fine-grid lookups use
// the absolute position rounded to float (the fine lists are registered
// against cells widened by 1e-5).
struct CylOrigin {
    float x, y, z;
};

__device__ __forceinline__ float cyl_dist_sq_local(const CylOrigin& G, float px, float py, float pz, float4 f) {
    if (f.x == 2.0f) {
        const float ez = (G.z - f.z) + pz, ey = (G.y - f.y) + py;
        return ez * ez + ey * ey;
    } else if (f.z == 2.0f) {
        const float ex = (G.x - f.x) + px, ey = (G.y - f.y) + py;
        return ex * ex + ey * ey;
    }
    const float ex = (G.x - f.x) + px, ez = (G.z - f.z) + pz;
    return ex * ex + ez * ez;
}

// Signs of d^2 - inR r^2 (in) and d^2 - r^2 (out).  Error of the FP32 d^2,
// u = 2^-24: a local coordinate e = (G - f) + p is off by at most
// u (|G - f| + |e|) <= u (2|e| + |p|) (two roundings); the squares and the sum
// add u d^2 each, so d^2 is off by at most u (6 d^2 + 2.83 |p| d), and the
// FP32 threshold inR r^2 by u inR r^2.  The band is 4x their sum at
// d^2 = max(inR r^2, r^2) = M.  nexact counts the FP64 decisions.
struct CylSides {
    int in, out;
};
__device__ __forceinline__ CylSides cyl_sides_local(const CylOrigin& G, float px, float py, float pz, float4 f,
                                                    float inR, uint32_t& ntests, uint32_t& nexact) {
    ntests++;
    const float cur = cyl_dist_sq_local(G, px, py, pz, f);
    const float A = inR * f.w, B = f.w;
    const float M = fmaxf(A, B);
    const float pm = fmaxf(fabsf(px), fmaxf(fabsf(py), fabsf(pz)));
    const float band = 2.4e-7f * (7.0f * M + 2.83f * pm * sqrtf(M));
    if (fabsf(cur - A) > band && fabsf(cur - B) > band) return {cur < A ? -1 : 1, cur < B ? -1 : 1};
    nexact++;
    const double c = cyl_dist_sq64((double)G.x + (double)px, (double)G.y + (double)py, (double)G.z + (double)pz, f);
    const double A64 = (double)inR * (double)f.w, B64 = (double)f.w;
    return {(int)(c > A64) - (int)(c < A64), (int)(c > B64) - (int)(c < B64)};
}

__device__ __forceinline__ void cyl_outside_entry_local(const CylOrigin& G, float4 f, const uint32_t* list,
                                                        uint32_t j, float ox, float oy, float oz, float& px,
                                                        float& py, float& pz, float u, float perm, float inR,
                                                        uint32_t& imo, uint32_t& nearest, uint32_t& nrej,
                                                        uint32_t& nperm, bool& moved, bool& inside,
                                                        uint32_t& ntests, uint32_t& nexact) {
    const CylSides s = cyl_sides_local(G, px, py, pz, f, inR, ntests, nexact);
    inside |= (s.in < 0) | (s.out < 0);
    if ((s.out <= 0) & (s.in > 0)) {
        if (u >= perm) { px = ox; py = oy; pz = oz; nrej++; moved = true; }
        else { imo = 1; nearest = __ldg(list + j); nperm++; }
    } else if (s.in < 0) {
        if (u < 1.0f - perm) { px = ox; py = oy; pz = oz; nrej++; moved = true; }
        else if ((1.0f - perm < u) & (u < 1.0f - perm * perm)) {
            px = ox; py = oy; pz = oz; nearest = __ldg(list + j); imo = 1; nrej++;
            moved = true;
        } else { imo = 0; nearest = __ldg(list + j); nperm++; }
    }
}

// cyl_membranes with local positions (origin G; o, p local to it) and the
// decisions of cyl_sides_local
__device__ __forceinline__ void cyl_membranes_local(const CylDev& g, const CylOrigin& G, float ox, float oy, float oz,
                                                    float& px, float& py, float& pz, float u, float perm, float inR,
                                                    uint32_t& imo, uint32_t& nearest, uint32_t& nrej,
                                                    uint32_t& nperm, uint32_t& status, uint32_t& ntests,
                                                    uint32_t& nexact) {
    if (!(perm < 1.0f)) return;
    if (imo < 2) {
        const float4 f = __ldg(g.fibers + nearest);
        const CylSides s = cyl_sides_local(G, px, py, pz, f, inR, ntests, nexact);
        if (imo == 0) {
            if ((s.in > 0) & (s.out <= 0)) {
                if (u >= perm) { px = ox; py = oy; pz = oz; nrej++; }
                else { imo = 1; nperm++; }
            } else if (s.out > 0) {
                if (u < 1.0f - perm) { px = ox; py = oy; pz = oz; nrej++; }
                else if ((1.0f - perm < u) & (u < 1.0f - perm * perm)) {
                    px = ox; py = oy; pz = oz; imo = 1; nrej++;
                } else { imo = 2; nperm++; }
            }
        } else {
            if (s.out > 0) {
                if (u >= perm) { px = ox; py = oy; pz = oz; nrej++; }
                else { imo = 2; nperm++; }
            } else if (s.in < 0) {
                if (u >= perm) { px = ox; py = oy; pz = oz; nrej++; }
                else { imo = 0; nperm++; }
            }
        }
        const CylSides e = cyl_sides_local(G, px, py, pz, f, inR, ntests, nexact);
        if (e.out > 0) imo = 2;
        else if (e.in < 0) imo = 0;
        else imo = 1;
        return;
    }
    uint32_t cube = cyl_cell(G.x + px, G.y + py, G.z + pz, g.L, g.n);
    uint32_t cnt = __ldg(g.cube_count + cube);
    const uint32_t* list = g.cubes + (size_t)cube * g.maxFPC;
    const float4* inl = g.cube_fibers ? g.cube_fibers + (size_t)cube * g.maxFPC : nullptr;
    bool moved = false, inside = false;
    const bool fine = g.fine_start != nullptr && inR <= 1.0f;
    uint32_t j = 0;
    if (fine) {
        const uint32_t fc = cyl_fine_cell(g, G.x + px, G.y + py, G.z + pz, cube);
        const uint32_t e1 = __ldg(g.fine_start + fc + 1);
        j = cnt;
        uint32_t jm = 0;
        for (uint32_t e = __ldg(g.fine_start + fc); e < e1; e++) {
            const uint32_t jj = __ldg(g.fine_pos + e);
            cyl_outside_entry_local(G, __ldg(g.fine_rec + e), list, jj, ox, oy, oz, px, py, pz, u, perm, inR, imo,
                                    nearest, nrej, nperm, moved, inside, ntests, nexact);
            if (moved) { jm = jj; break; }
        }
        if (moved) {
            if (cyl_cell(G.x + px, G.y + py, G.z + pz, g.L, g.n) == cube) {
                const uint32_t fo = cyl_fine_cell(g, G.x + px, G.y + py, G.z + pz, cube);
                const uint32_t eo1 = __ldg(g.fine_start + fo + 1);
                for (uint32_t e = __ldg(g.fine_start + fo); e < eo1; e++) {
                    const uint32_t jj = __ldg(g.fine_pos + e);
                    if (jj <= jm) continue;
                    cyl_outside_entry_local(G, __ldg(g.fine_rec + e), list, jj, ox, oy, oz, px, py, pz, u, perm,
                                            inR, imo, nearest, nrej, nperm, moved, inside, ntests, nexact);
                }
            } else {
                j = jm + 1;
            }
        }
    }
    for (; j < cnt; j++) {
        float4 f;
        if (inl) {
            f = __ldg(inl + j);
        } else {
            const uint32_t fi = __ldg(list + j);
            if (fi >= g.nF) { status |= kStatusBadCell; continue; }
            f = __ldg(g.fibers + fi);
        }
        cyl_outside_entry_local(G, f, list, j, ox, oy, oz, px, py, pz, u, perm, inR, imo, nearest, nrej, nperm,
                                moved, inside, ntests, nexact);
    }
    if (imo == 2 && (moved || inside)) {
        cube = cyl_cell(G.x + px, G.y + py, G.z + pz, g.L, g.n);
        cnt = __ldg(g.cube_count + cube);
        list = g.cubes + (size_t)cube * g.maxFPC;
        inl = g.cube_fibers ? g.cube_fibers + (size_t)cube * g.maxFPC : nullptr;
        if (fine && moved) {
            const uint32_t fc = cyl_fine_cell(g, G.x + px, G.y + py, G.z + pz, cube);
            const uint32_t e1 = __ldg(g.fine_start + fc + 1);
            for (uint32_t e = __ldg(g.fine_start + fc); e < e1; e++) {
                const CylSides s = cyl_sides_local(G, px, py, pz, __ldg(g.fine_rec + e), inR, ntests, nexact);
                if ((s.in < 0) | (s.out < 0)) { px = ox; py = oy; pz = oz; nrej++; }
            }
        } else {
            for (uint32_t j2 = 0; j2 < cnt; j2++) {
                float4 f;
                if (inl) {
                    f = __ldg(inl + j2);
                } else {
                    const uint32_t fi = __ldg(list + j2);
                    if (fi >= g.nF) { status |= kStatusBadCell; continue; }
                    f = __ldg(g.fibers + fi);
                }
                const CylSides s = cyl_sides_local(G, px, py, pz, f, inR, ntests, nexact);
                if ((s.in < 0) | (s.out < 0)) { px = ox; py = oy; pz = oz; nrej++; }
            }
        }
    }
}

}  // namespace dsim
