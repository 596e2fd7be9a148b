/*
 * oracle_dsim2.c -- CPU restatement of the dSim2 (infinite cylinder) hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU cylinder engine.
 * Compile with -ffp-contract=off.  Expression order follows the reference
 * (rfdougherty/dSim, dSim2/src/) so results are bit-identical to its CPU path.
 */
#include "oracle.h"
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define HALO 1.1f          /* HALO_DISTANCE, dSim2/src/options.h:10 */
#define MAX_GRID 100u      /* MAX_GRID_SIZE, dSim2/src/options.h:7  */

/* float -> uint as the reference's x86-64 build converts it (the value
 * 4294967296.0f, i.e. (float)UINT_MAX, comes back as 0). */
static inline uint32_t f2u(float x) {
    return (x >= 4294967296.0f) ? 0u : (uint32_t)x;
}

/* initFibers(FILE*), dSim2/src/spinSystem.cpp:323-385 */
int or2_load_fibers(const char* path, float spaceScale, float* fiberPos, float* maxR) {
    FILE* fp = fopen(path, "r");
    if (!fp) return -1;
    char str[256];
    float x, y, z, r;
    int n = 0;
    float mr = 0.0f;
    while (fgets(str, 255, fp) != NULL) {
        if (sscanf(str, "%f %f %f %f", &x, &y, &z, &r) == 4 &&
            (fabsf(x) + r < spaceScale || x == INFINITY) &&
            (fabsf(y) + r < spaceScale || y == INFINITY) &&
            (fabsf(z) + r < spaceScale || z == INFINITY) && r > 0) {
            if (fiberPos) {
                r = r / spaceScale;
                if (r > mr) mr = r;
                x = x / spaceScale; if (x > 2.0 || x == INFINITY) x = 2.0f;
                y = y / spaceScale; if (y > 2.0 || y == INFINITY) y = 2.0f;
                z = z / spaceScale; if (z > 2.0 || z == INFINITY) z = 2.0f;
                fiberPos[4 * n + 0] = x;
                fiberPos[4 * n + 1] = y;
                fiberPos[4 * n + 2] = z;
                fiberPos[4 * n + 3] = r * r;
            }
            n++;
        }
    }
    fclose(fp);
    if (maxR) *maxR = mr;
    return n;
}

/* calcCubePos/calcCubeHash, dSim2/src/spinSystem.cpp:413-433.  The float3
 * division of the reference's header multiplies by the reciprocal. */
static inline int cube_hash2(float px, float py, float pz, float L, uint32_t n) {
    float inv = 1.0f / L;
    float cx = floorf((px + 1.0f) * inv);
    float cy = floorf((py + 1.0f) * inv);
    float cz = floorf((pz + 1.0f) * inv);
    float hi = (float)(n - 1);
    cx = fmaxf(fminf(cx, hi), 0.0f);
    cy = fmaxf(fminf(cy, hi), 0.0f);
    cz = fmaxf(fminf(cz, hi), 0.0f);
    return (int)((float)(n * n) * cz) + (int)((float)n * cy) + (int)cx;
}
static inline void cube_pos2(float p[3], float L, float out[3]) {
    float inv = 1.0f / L;
    out[0] = floorf((p[0] + 1.0f) * inv);
    out[1] = floorf((p[1] + 1.0f) * inv);
    out[2] = floorf((p[2] + 1.0f) * inv);
}

typedef struct {
    uint32_t n, maxFPC;
    float L, maxR;
    uint32_t* cc;
    uint32_t* cubes;
} grid2;

/* FILL_LIST_{X,Y,Z}, dSim2/src/spinSystem.cpp:448-481: walk the fiber axis */
static void fill_line(grid2* g, float cp[3], int axis, uint32_t fib) {
    cp[axis] = (float)(-1 + 0.002);
    for (uint32_t j = 0; j < g->n; j++) {
        int index = cube_hash2(cp[0], cp[1], cp[2], g->L, g->n);
        uint32_t counter = g->cc[index];
        g->cc[index] += 1;
        if (g->cubes) g->cubes[(size_t)index * g->maxFPC + counter] = fib;
        cp[axis] += g->L;
    }
}

/* addEntities, dSim2/src/spinSystem.cpp:483-745.  For a fiber along `a`,
 * the halo first tests axis `f` (with neighbours along `s`), then axis `s`. */
static void add_fiber(grid2* g, const float* fp, uint32_t fib, int a, int f, int s) {
    float cp[3] = {fp[0], fp[1], fp[2]};
    fill_line(g, cp, a, fib);
    float tp[3] = {fp[0], fp[1], fp[2]};
    tp[a] = (float)(-1 + 0.002);
    float cpos[3];
    cube_pos2(tp, g->L, cpos);
    float dfc_f = tp[f] - cpos[f] * g->L;
    float dfc_s = tp[s] - cpos[s] * g->L;
    float H = HALO * g->maxR;
    if (dfc_f < H) {
        cp[f] -= H;
        if (cp[f] > -1) {
            fill_line(g, cp, a, fib);
            if ((cp[s] - g->L) > -1) { cp[s] -= g->L; fill_line(g, cp, a, fib); cp[s] += g->L; }
            if ((cp[s] + g->L) < 1) { cp[s] += g->L; fill_line(g, cp, a, fib); cp[s] -= g->L; }
        }
        cp[f] += H;
    } else if (dfc_f > (g->L - H)) {
        cp[f] += H;
        if (cp[f] < 1) {
            fill_line(g, cp, a, fib);
            if ((cp[s] - g->L) > -1) { cp[s] -= g->L; fill_line(g, cp, a, fib); cp[s] += g->L; }
            if ((cp[s] + g->L) < 1) { cp[s] += g->L; fill_line(g, cp, a, fib); cp[s] -= g->L; }
        }
        cp[f] -= H;
    }
    if (dfc_s < H) {
        if ((cp[s] - g->L) > -1) { cp[s] -= g->L; fill_line(g, cp, a, fib); cp[s] += g->L; }
    } else if (dfc_s > (g->L - H)) {
        if ((cp[s] + g->L) < 1) { cp[s] += g->L; fill_line(g, cp, a, fib); cp[s] -= g->L; }
    }
}

/* build() :135-228 (grid geometry) + addEntities() */
int or2_build_grid(uint32_t nF, const float* fiberPos, float maxR, uint32_t geom[2],
                   float* cubeLength, uint32_t* cubeCounter, uint32_t* cubes) {
    uint32_t t = (uint32_t)(2.0f / (float)(maxR * 4)) - 1;
    if (t < 2) t = 2;
    if (t > MAX_GRID) t = MAX_GRID;
    uint32_t n = t;
    uint32_t maxFPC = (uint32_t)ceil((double)(nF / (n * n) * 10));
    float L = 2.0f / n;
    geom[0] = n; geom[1] = maxFPC;
    *cubeLength = L;
    if (!cubeCounter) return 0;
    grid2 g = {n, maxFPC, L, maxR, cubeCounter, cubes};
    size_t total = (size_t)n * n * n;
    memset(cubeCounter, 0, total * sizeof(uint32_t));
    /* a counting pass first so that an overflowing cell never writes out of
     * bounds (the reference writes past the cell, then fails in build()) */
    grid2 gc = g; gc.cubes = NULL;
    for (uint32_t i = 0; i < nF; i++) {
        const float* fp = fiberPos + 4 * (size_t)i;
        if (fp[0] == 2.0f) add_fiber(&gc, fp, i, 0, 2, 1);
        else if (fp[2] == 2.0f) add_fiber(&gc, fp, i, 2, 0, 1);
        else if (fp[1] == 2.0f) add_fiber(&gc, fp, i, 1, 2, 0);
    }
    uint32_t maxE = 0;
    for (size_t c = 0; c < total; c++) if (cubeCounter[c] > maxE) maxE = cubeCounter[c];
    if (maxE > maxFPC) return -1;
    memset(cubeCounter, 0, total * sizeof(uint32_t));
    for (uint32_t i = 0; i < nF; i++) {
        const float* fp = fiberPos + 4 * (size_t)i;
        if (fp[0] == 2.0f) add_fiber(&g, fp, i, 0, 2, 1);
        else if (fp[2] == 2.0f) add_fiber(&g, fp, i, 2, 0, 1);
        else if (fp[1] == 2.0f) add_fiber(&g, fp, i, 1, 2, 0);
    }
    return 0;
}

/* distToCenterSq, dSim2/src/spinKernelCpu.cpp:71-82 */
static inline float dist_sq(float px, float py, float pz, const float* f) {
    if (f[0] == 2.0f) return (pz - f[2]) * (pz - f[2]) + (py - f[1]) * (py - f[1]);
    else if (f[2] == 2.0f) return (px - f[0]) * (px - f[0]) + (py - f[1]) * (py - f[1]);
    return (px - f[0]) * (px - f[0]) + (pz - f[2]) * (pz - f[2]);
}

/* findNearestFiber, dSim2/src/spinSystem.cpp:1223-1311 */
void or2_find_nearest(uint32_t N, const float* pos4, const float* fiberPos, uint32_t numCubes,
                      float cubeLength, uint32_t maxFPC, const uint32_t* cc, const uint32_t* cubes,
                      float innerRadiusProportion, uint32_t* nearest, uint32_t* imoOut) {
    float inRadPropSq = innerRadiusProportion * innerRadiusProportion;
    for (uint32_t s = 0; s < N; s++) {
        uint32_t imo = 2;
        int nearestTube = -1;
        float px = pos4[4 * s], py = pos4[4 * s + 1], pz = pos4[4 * s + 2];
        float minD = 9.9e9f;
        for (int dy = -1; dy <= 1; dy++) {
            float ty = py + dy * cubeLength;
            if (fabsf(ty) <= 1) {
                for (int dx = -1; dx <= 1; dx++) {
                    float tx = px + dx * cubeLength;
                    if (fabsf(tx) <= 1) {
                        for (int dz = -1; dz <= 1; dz++) {
                            float tz = pz + dz * cubeLength;
                            if (fabsf(tz) <= 1) {
                                uint32_t cube = (uint32_t)cube_hash2(tx, ty, tz, cubeLength, numCubes);
                                for (uint32_t j = 0; j < cc[cube]; j++) {
                                    int i = (int)cubes[(size_t)cube * maxFPC + j];
                                    const float* f = fiberPos + 4 * (size_t)i;
                                    float radSq = f[3];
                                    float d = dist_sq(px, py, pz, f);
                                    if (d < radSq) imo = (d < inRadPropSq * radSq) ? 0u : 1u;
                                    if (d < minD) { nearestTube = i; minD = d; }
                                }
                            }
                        }
                    }
                }
            }
        }
        nearest[s] = (uint32_t)nearestTube;
        imoOut[s] = imo;
    }
}

/* cpuIntegrate, dSim2/src/spinKernelCpu.cpp:312-641 (draws replace myRandn at :358) */
static void step2(const or2_params* P, uint32_t idx, float* pos4, uint32_t* seed4, float* pp,
                  const float* FP, const uint32_t* cc, const uint32_t* cubes, float gx, float gy,
                  float gz, float pc, float intraSd, float extraSd, float myelinSd,
                  float inRadPropSq, const float d[4], uint32_t* cnt) {
    float* P5 = pp + 5 * (size_t)idx;
    float ox = pos4[4 * idx], oy = pos4[4 * idx + 1], oz = pos4[4 * idx + 2];
    float px = ox, py = oy, pz = oz;
    uint32_t nearest = f2u(P5[2]);
    uint32_t imo = f2u(P5[3]);
    float u = d[3];
    float sd = (imo == 0) ? intraSd : ((imo == 1) ? myelinSd : extraSd);
    px += d[0] * sd;
    py += d[1] * sd;
    pz += d[2] * sd;
    float perm = P->permeability;
    if (perm < 1.0f) {
        float radSq, cur;
        if (imo < 2) {
            const float* f = FP + 4 * (size_t)nearest;
            radSq = f[3];
            cur = dist_sq(px, py, pz, f);
            if (imo == 0) {
                if ((cur > inRadPropSq * radSq) & (cur <= radSq)) {
                    if (u >= perm) { px = ox; py = oy; pz = oz; if (cnt) cnt[0]++; }
                    else { imo = 1; if (cnt) cnt[1]++; }
                } else if (cur > radSq) {
                    if (u < 1 - perm) { px = ox; py = oy; pz = oz; if (cnt) cnt[0]++; }
                    else if ((1 - perm < u) & (u < 1 - perm * perm)) {
                        px = ox; py = oy; pz = oz; imo = 1; if (cnt) cnt[0]++;
                    } else { imo = 2; if (cnt) cnt[1]++; }
                }
            } else {
                if (cur > radSq) {
                    if (u >= perm) { px = ox; py = oy; pz = oz; if (cnt) cnt[0]++; }
                    else { imo = 2; if (cnt) cnt[1]++; }
                } else if (cur < inRadPropSq * radSq) {
                    if (u >= perm) { px = ox; py = oy; pz = oz; if (cnt) cnt[0]++; }
                    else { imo = 0; if (cnt) cnt[1]++; }
                }
            }
            float endD = dist_sq(px, py, pz, f);
            if (endD > radSq) imo = 2;
            else if (endD < inRadPropSq * radSq) imo = 0;
            else imo = 1;
        } else {
            uint32_t cube = (uint32_t)cube_hash2(px, py, pz, P->cubeLength, P->numCubes);
            for (uint32_t j = 0; j < cc[cube]; j++) {
                uint32_t i = cubes[(size_t)cube * P->maxFibersPerCube + j];
                const float* f = FP + 4 * (size_t)i;
                radSq = f[3];
                cur = dist_sq(px, py, pz, f);
                if ((cur <= radSq) & (cur > inRadPropSq * radSq)) {
                    if (u >= perm) { px = ox; py = oy; pz = oz; if (cnt) cnt[0]++; }
                    else { imo = 1; nearest = i; if (cnt) cnt[1]++; }
                } else if (cur < inRadPropSq * radSq) {
                    if (u < 1 - perm) { px = ox; py = oy; pz = oz; if (cnt) cnt[0]++; }
                    else if ((1 - perm < u) & (u < 1 - perm * perm)) {
                        px = ox; py = oy; pz = oz; nearest = i; imo = 1; if (cnt) cnt[0]++;
                    } else { imo = 0; nearest = i; if (cnt) cnt[1]++; }
                }
            }
            /* second pass: a spin that bounced into another fiber, :560-589 */
            cube = (uint32_t)cube_hash2(px, py, pz, P->cubeLength, P->numCubes);
            if (imo == 2) {
                for (uint32_t j = 0; j < cc[cube]; j++) {
                    uint32_t i = cubes[(size_t)cube * P->maxFibersPerCube + j];
                    const float* f = FP + 4 * (size_t)i;
                    radSq = f[3];
                    float nd = dist_sq(px, py, pz, f);
                    if (nd < inRadPropSq * radSq) { px = ox; py = oy; pz = oz; if (cnt) cnt[0]++; }
                    else if (nd < radSq) { px = ox; py = oy; pz = oz; if (cnt) cnt[0]++; }
                }
            }
        }
    }
    float sr = P->spinRadius;
    if (px > 1.0f - sr) { px = 1.0f - sr; } else if (px < -1.0f + sr) { px = -1.0f + sr; }
    if (py > 1.0f - sr) { py = 1.0f - sr; } else if (py < -1.0f + sr) { py = -1.0f + sr; }
    if (pz > 1.0f - sr) { pz = 1.0f - sr; } else if (pz < -1.0f + sr) { pz = -1.0f + sr; }
    pos4[4 * idx] = px; pos4[4 * idx + 1] = py; pos4[4 * idx + 2] = pz;
    float dt = P->deltaTime;
    switch (imo) {
        case 0: P5[0] += -P5[0] / P->T2fiber * dt; break;
        case 1: P5[0] += -P5[0] / P->T2myelin * dt; break;
        case 2: P5[0] += -P5[0] / P->T2outside * dt; break;
    }
    P5[1] += (gx * px + gy * py + gz * pz) * pc;
    P5[2] = (float)nearest;
    P5[3] = (float)imo;
    seed4[4 * idx + 3] = nearest;
}

void or2_integrate(const or2_params* P, uint32_t N, float* pos4, uint32_t* seed4, float* params5,
                   const float* fiberPos, const uint32_t* cc, const uint32_t* cubes, float gx,
                   float gy, float gz, float phaseConstant, uint32_t iterations, const float* draws,
                   float* drawsOut, uint32_t* counts) {
    float dt = P->deltaTime;
    for (uint32_t it = 0; it < iterations; it++) {
        /* cpuIntegrateSystem, dSim2/src/spinKernelCpu.cpp:2-20 */
        float intraSd = sqrtf(2.0f * P->intraAdcScaled * dt);
        float extraSd = sqrtf(2.0f * P->extraAdcScaled * dt);
        float myelinSd = sqrtf(2.0f * P->myelinAdcScaled * dt);
        float inRadPropSq = P->innerRadiusProportion * P->innerRadiusProportion;
        for (uint32_t i = 0; i < N; i++) {
            float d[4];
            if (draws) {
                const float* src = draws + ((size_t)it * N + i) * 4;
                d[0] = src[0]; d[1] = src[1]; d[2] = src[2]; d[3] = src[3];
            } else {
                uint32_t s[2] = {seed4[4 * i], seed4[4 * i + 1]};
                or_myrandn(s, d);
                seed4[4 * i] = s[0]; seed4[4 * i + 1] = s[1];
            }
            if (drawsOut) memcpy(drawsOut + ((size_t)it * N + i) * 4, d, sizeof(d));
            step2(P, i, pos4, seed4, params5, fiberPos, cc, cubes, gx, gy, gz, phaseConstant,
                  intraSd, extraSd, myelinSd, inRadPropSq, d, counts ? counts + 2 * (size_t)i : NULL);
        }
    }
}

/* getMrSignal(), dSim2/src/spinSystem.cpp:944-978 */
double or2_signal(uint32_t N, const float* pos4, const float* params5) {
    double X = 0, Y = 0;
    double dlim = 0.80f;
    uint32_t n = 0;
    for (uint32_t i = 0; i < N; i++) {
        const float* p = pos4 + 4 * (size_t)i;
        const float* q = params5 + 5 * (size_t)i;
        if (p[0] > -dlim && p[0] < dlim && p[1] > -dlim && p[1] < dlim && p[2] > -dlim && p[2] < dlim) {
            X += (double)(cosf(q[1]) * q[0]);
            Y += (double)(sinf(q[1]) * q[0]);
            n++;
        }
    }
    return sqrt(X * X + Y * Y) / (double)n;
}

void or2_integrate_multi(const or2_params* P, uint32_t N, float* pos4, uint32_t* seed4, float* params5,
                         const float* fiberPos, const uint32_t* cc, const uint32_t* cubes, uint32_t nG,
                         const float* grads, const float* wave, float phaseConstant, uint32_t iterations,
                         const float* draws, float* phases, uint32_t* counts, int nthreads) {
    float dt = P->deltaTime;
    /* cpuIntegrateSystem, dSim2/src/spinKernelCpu.cpp:2-20 */
    float intraSd = sqrtf(2.0f * P->intraAdcScaled * dt);
    float extraSd = sqrtf(2.0f * P->extraAdcScaled * dt);
    float myelinSd = sqrtf(2.0f * P->myelinAdcScaled * dt);
    float inRadPropSq = P->innerRadiusProportion * P->innerRadiusProportion;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (uint32_t i = 0; i < N; i++) {
        float* ph = phases + (size_t)i * nG;
        for (uint32_t it = 0; it < iterations; it++) {
            float d[4];
            if (draws) {
                const float* src = draws + ((size_t)it * N + i) * 4;
                d[0] = src[0]; d[1] = src[1]; d[2] = src[2]; d[3] = src[3];
            } else {
                uint32_t s[2] = {seed4[4 * i], seed4[4 * i + 1]};
                or_myrandn(s, d);
                seed4[4 * i] = s[0]; seed4[4 * i + 1] = s[1];
            }
            step2(P, i, pos4, seed4, params5, fiberPos, cc, cubes, 0.0f, 0.0f, 0.0f, phaseConstant, intraSd,
                  extraSd, myelinSd, inRadPropSq, d, counts ? counts + 2 * (size_t)i : NULL);
            const float w = wave[it];
            const float* q = pos4 + 4 * (size_t)i;
            for (uint32_t k = 0; k < nG; k++) {
                float gx = w * grads[3 * k], gy = w * grads[3 * k + 1], gz = w * grads[3 * k + 2];
                ph[k] += (gx * q[0] + gy * q[1] + gz * q[2]) * phaseConstant;
            }
        }
    }
}

/* ---- FP64 restatement (precision oracle for cylinders) ---------------------
 * step2 with every position-dependent quantity in double: the proposed step,
 * the distances to the fibers (fiberPos promoted), the clamp, T2 decay and
 * the phases.  Same rules and branch order as cpuIntegrate
 * (dSim2/src/spinKernelCpu.cpp:312-641); the draws are the same float stream
 * as the FP32 walk's. */
static inline double dist_sq_f64(double px, double py, double pz, const float* f) {
    const double fx = f[0], fy = f[1], fz = f[2];
    if (f[0] == 2.0f) return (pz - fz) * (pz - fz) + (py - fy) * (py - fy);
    else if (f[2] == 2.0f) return (px - fx) * (px - fx) + (py - fy) * (py - fy);
    return (px - fx) * (px - fx) + (pz - fz) * (pz - fz);
}

/* calcCubePos/calcCubeHash in double, multiplying by the reciprocal as the
 * reference's float3 division does (cube_hash2 above) */
static inline uint32_t cube_hash2_f64(double px, double py, double pz, float L, uint32_t n) {
    double inv = 1.0 / (double)L;
    double hi = (double)(n - 1);
    double cx = fmax(fmin(floor((px + 1.0) * inv), hi), 0.0);
    double cy = fmax(fmin(floor((py + 1.0) * inv), hi), 0.0);
    double cz = fmax(fmin(floor((pz + 1.0) * inv), hi), 0.0);
    return (uint32_t)cz * n * n + (uint32_t)cy * n + (uint32_t)cx;
}

static void step2_f64(const or2_params* P, double* q, double* mag, uint32_t* imoP, uint32_t* nearP,
                      const float* FP, const uint32_t* cc, const uint32_t* cubes, double intraSd,
                      double extraSd, double myelinSd, double inRadPropSq, const float d[4]) {
    double ox = q[0], oy = q[1], oz = q[2];
    double px = ox, py = oy, pz = oz;
    uint32_t nearest = *nearP, imo = *imoP;
    double u = d[3];
    double sd = (imo == 0) ? intraSd : ((imo == 1) ? myelinSd : extraSd);
    px += (double)d[0] * sd;
    py += (double)d[1] * sd;
    pz += (double)d[2] * sd;
    double perm = P->permeability;
    if (perm < 1.0) {
        double radSq, cur;
        if (imo < 2) {
            const float* f = FP + 4 * (size_t)nearest;
            radSq = f[3];
            cur = dist_sq_f64(px, py, pz, f);
            if (imo == 0) {
                if ((cur > inRadPropSq * radSq) & (cur <= radSq)) {
                    if (u >= perm) { px = ox; py = oy; pz = oz; }
                    else { imo = 1; }
                } else if (cur > radSq) {
                    if (u < 1 - perm) { px = ox; py = oy; pz = oz; }
                    else if ((1 - perm < u) & (u < 1 - perm * perm)) { px = ox; py = oy; pz = oz; imo = 1; }
                    else { imo = 2; }
                }
            } else {
                if (cur > radSq) {
                    if (u >= perm) { px = ox; py = oy; pz = oz; }
                    else { imo = 2; }
                } else if (cur < inRadPropSq * radSq) {
                    if (u >= perm) { px = ox; py = oy; pz = oz; }
                    else { imo = 0; }
                }
            }
            double endD = dist_sq_f64(px, py, pz, f);
            if (endD > radSq) imo = 2;
            else if (endD < inRadPropSq * radSq) imo = 0;
            else imo = 1;
        } else {
            uint32_t cube = cube_hash2_f64(px, py, pz, P->cubeLength, P->numCubes);
            for (uint32_t j = 0; j < cc[cube]; j++) {
                uint32_t i = cubes[(size_t)cube * P->maxFibersPerCube + j];
                const float* f = FP + 4 * (size_t)i;
                radSq = f[3];
                cur = dist_sq_f64(px, py, pz, f);
                if ((cur <= radSq) & (cur > inRadPropSq * radSq)) {
                    if (u >= perm) { px = ox; py = oy; pz = oz; }
                    else { imo = 1; nearest = i; }
                } else if (cur < inRadPropSq * radSq) {
                    if (u < 1 - perm) { px = ox; py = oy; pz = oz; }
                    else if ((1 - perm < u) & (u < 1 - perm * perm)) { px = ox; py = oy; pz = oz; nearest = i; imo = 1; }
                    else { imo = 0; nearest = i; }
                }
            }
            cube = cube_hash2_f64(px, py, pz, P->cubeLength, P->numCubes);
            if (imo == 2) {
                for (uint32_t j = 0; j < cc[cube]; j++) {
                    uint32_t i = cubes[(size_t)cube * P->maxFibersPerCube + j];
                    const float* f = FP + 4 * (size_t)i;
                    radSq = f[3];
                    double nd = dist_sq_f64(px, py, pz, f);
                    if (nd < inRadPropSq * radSq) { px = ox; py = oy; pz = oz; }
                    else if (nd < radSq) { px = ox; py = oy; pz = oz; }
                }
            }
        }
    }
    double sr = P->spinRadius;
    if (px > 1.0 - sr) { px = 1.0 - sr; } else if (px < -1.0 + sr) { px = -1.0 + sr; }
    if (py > 1.0 - sr) { py = 1.0 - sr; } else if (py < -1.0 + sr) { py = -1.0 + sr; }
    if (pz > 1.0 - sr) { pz = 1.0 - sr; } else if (pz < -1.0 + sr) { pz = -1.0 + sr; }
    q[0] = px; q[1] = py; q[2] = pz;
    double dt = P->deltaTime;
    switch (imo) {
        case 0: *mag += -*mag / (double)P->T2fiber * dt; break;
        case 1: *mag += -*mag / (double)P->T2myelin * dt; break;
        case 2: *mag += -*mag / (double)P->T2outside * dt; break;
    }
    *imoP = imo;
    *nearP = nearest;
}

void or2_integrate_f64_multi(const or2_params* P, uint32_t N, double* pos3, double* mag, uint32_t* imo,
                             uint32_t* nearest, const float* fiberPos, const uint32_t* cc, const uint32_t* cubes,
                             uint32_t nG, const double* grads, const double* wave, double phaseConstant,
                             uint32_t iterations, const float* draws, double* phases, int nthreads) {
    /* the parameters are the reference's float values (sigma as
     * cpuIntegrateSystem computes it, dSim2/src/spinKernelCpu.cpp:2-20);
     * the walk is in double */
    float fdt = P->deltaTime;
    double intraSd = sqrtf(2.0f * P->intraAdcScaled * fdt);
    double extraSd = sqrtf(2.0f * P->extraAdcScaled * fdt);
    double myelinSd = sqrtf(2.0f * P->myelinAdcScaled * fdt);
    double inRadPropSq = P->innerRadiusProportion * P->innerRadiusProportion;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (uint32_t i = 0; i < N; i++) {
        double* q = pos3 + 3 * (size_t)i;
        double* ph = phases + (size_t)i * nG;
        for (uint32_t it = 0; it < iterations; it++) {
            step2_f64(P, q, mag + i, imo + i, nearest + i, fiberPos, cc, cubes, intraSd, extraSd, myelinSd,
                      inRadPropSq, draws + ((size_t)it * N + i) * 4);
            const double w = wave[it];
            if (w == 0.0) continue;
            for (uint32_t k = 0; k < nG; k++)
                ph[k] += w * (grads[3 * k] * q[0] + grads[3 * k + 1] * q[1] + grads[3 * k + 2] * q[2]) * phaseConstant;
        }
    }
}
