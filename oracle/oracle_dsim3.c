/*
 * oracle_dsim3.c -- CPU restatement of the dSim3 (triangle-mesh) hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU engine, never the product.
 * Compile with -ffp-contract=off so every float expression rounds exactly as
 * the reference's x86-64 build does (no FMA contraction, FLT_EVAL_METHOD 0).
 *
 * Each function cites the reference function it restates (paths inside
 * rfdougherty/dSim).  Expression order inside every float expression follows
 * the reference so results are bit-identical.
 */
#include "oracle.h"
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define OR_TWOPI 6.28318530717959f  /* dSim3/src/spinSystem.cpp:20 */

typedef struct { float x, y, z; } f3;
static inline f3 mk(float x, float y, float z) { f3 r = {x, y, z}; return r; }

/* ------------------------------------------------------------------------ */
/* MWC + Box-Muller: dSim3/src/spinKernelCpu.cpp:27-63                        */
/* ------------------------------------------------------------------------ */
static inline uint32_t mwc(uint32_t s[2]) {
    s[0] = 36969u * (s[0] & 65535u) + (s[0] >> 16);
    s[1] = 18000u * (s[1] & 65535u) + (s[1] >> 16);
    return (s[0] << 16) + s[1];
}
static inline void box_muller(float* u1, float* u2) {
    float r = sqrtf(-2.0f * logf(*u1));
    float phi = OR_TWOPI * *u2;
    *u1 = r * cosf(phi);
    *u2 = r * sinf(phi);
}
void or_myrandn(uint32_t seed[2], float out[4]) {
    float n1 = ((float)mwc(seed) + 1.0f) / 4294967296.0f;
    float n2 = ((float)mwc(seed) + 1.0f) / 4294967296.0f;
    float n3 = ((float)mwc(seed) + 1.0f) / 4294967296.0f;
    float u = ((float)mwc(seed) + 1.0f) / 4294967296.0f;
    float n4 = u;
    box_muller(&n1, &n2);
    box_muller(&n3, &n4);
    out[0] = n1; out[1] = n2; out[2] = n3; out[3] = u;
}

/* ------------------------------------------------------------------------ */
/* Philox4x32-10, restated from Salmon, Moraes, Dror, Shaw, "Parallel random */
/* numbers: as easy as 1, 2, 3" (SC'11): round multipliers, Weyl key bumps.  */
/* ------------------------------------------------------------------------ */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0; c1 = lo1; c2 = hi0 ^ c3 ^ k1; c3 = lo0;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* ------------------------------------------------------------------------ */
/* Mesh file parser: SpinSystem::initFibers, dSim3/src/spinSystem.cpp:290-673 */
/* Two passes over the file with the same fscanf grammar: a single character */
/* selects the block (V, T, A<k>, M<k>, G<k>), numbers follow until a scan    */
/* fails.  Pass one counts, pass two fills.                                  */
/* ------------------------------------------------------------------------ */
static int mesh_pass(FILE* fp, int fill, float spaceScale, uint32_t counts[7],
                     float* vertices, uint32_t* trgls, uint32_t* triInfo, float maxabs[3]) {
    char dataType = 'X';
    int nScanned;
    uint32_t i;
    float x, y, z, v1, v2, v3, nr, tri;
    while (!feof(fp)) {
        nScanned = fscanf(fp, "%c", &dataType);
        (void)nScanned;
        if (dataType == 'V') {
            i = 0; nScanned = 3;
            while (nScanned == 3) {
                nScanned = fscanf(fp, "%g %g %g", &x, &y, &z);
                if (nScanned == 3) {
                    if (!fill) counts[0]++;
                    else {
                        vertices[i * 3 + 0] = x / spaceScale;
                        vertices[i * 3 + 1] = y / spaceScale;
                        vertices[i * 3 + 2] = z / spaceScale;
                        maxabs[0] = fmaxf(fabsf(x) / spaceScale, maxabs[0]);
                        maxabs[1] = fmaxf(fabsf(y) / spaceScale, maxabs[1]);
                        maxabs[2] = fmaxf(fabsf(z) / spaceScale, maxabs[2]);
                        i++;
                    }
                }
            }
        } else if (dataType == 'T') {
            i = 0; nScanned = 3;
            while (nScanned == 3) {
                nScanned = fscanf(fp, "%g %g %g", &v1, &v2, &v3);
                if (nScanned == 3) {
                    if (!fill) counts[1]++;
                    else {
                        trgls[i * 3 + 0] = (uint32_t)v1;
                        trgls[i * 3 + 1] = (uint32_t)v2;
                        trgls[i * 3 + 2] = (uint32_t)v3;
                        triInfo[i * 3 + 2] = (uint32_t)v1;
                        i++;
                    }
                }
            }
        } else if (dataType == 'A' || dataType == 'M' || dataType == 'G') {
            uint32_t membrane = dataType == 'A' ? 0u : (dataType == 'M' ? 1u : 2u);
            if (!fill) counts[3 + membrane]++;
            nScanned = fscanf(fp, "%g", &nr);
            nScanned = 1; i = 0;
            while (nScanned == 1) {
                nScanned = fscanf(fp, "%g", &tri);
                if (nScanned == 1) {
                    if (fill) {
                        triInfo[(uint32_t)tri * 3] = (uint32_t)nr;
                        triInfo[(uint32_t)tri * 3 + 1] = membrane;
                    }
                    i++;
                }
            }
            if (!fill && i > counts[6]) counts[6] = i;
        }
    }
    return 0;
}

int or3_mesh_count(const char* path, uint32_t counts[7]) {
    FILE* fp = fopen(path, "r");
    if (!fp) return -1;
    memset(counts, 0, 7 * sizeof(uint32_t));
    mesh_pass(fp, 0, 1.0f, counts, NULL, NULL, NULL, NULL);
    fclose(fp);
    counts[2] = counts[3] + counts[5];  /* m_nFibers = m_nAxonFibers + m_nGliaFibers */
    if (counts[3] != counts[4]) return -2;
    return 0;
}

int or3_mesh_fill(const char* path, float spaceScale, const uint32_t counts[7],
                  float* vertices, uint32_t* trgls, uint32_t* triInfo,
                  float* helpers, float maxabs[3]) {
    FILE* fp = fopen(path, "r");
    if (!fp) return -1;
    uint32_t c[7];
    memcpy(c, counts, sizeof(c));
    memset(triInfo, 0, (size_t)counts[1] * 3 * sizeof(uint32_t));
    maxabs[0] = maxabs[1] = maxabs[2] = 1.0f;  /* m_xmax = m_ymax = m_zmax = 1.0f (ctor :72) */
    mesh_pass(fp, 1, spaceScale, c, vertices, trgls, triInfo, maxabs);
    fclose(fp);
    /* m_triangleHelpers, spinSystem.cpp:612-648 */
    for (uint32_t t = 0; t < counts[1]; t++) {
        uint32_t p1 = trgls[t * 3 + 0], p2 = trgls[t * 3 + 1], p3 = trgls[t * 3 + 2];
        float x1 = vertices[p1 * 3 + 0], y1 = vertices[p1 * 3 + 1], z1 = vertices[p1 * 3 + 2];
        float x2 = vertices[p2 * 3 + 0], y2 = vertices[p2 * 3 + 1], z2 = vertices[p2 * 3 + 2];
        float x3 = vertices[p3 * 3 + 0], y3 = vertices[p3 * 3 + 1], z3 = vertices[p3 * 3 + 2];
        float nx = (y2 - y1) * (z3 - z1) - (z2 - z1) * (y3 - y1);
        float ny = (z2 - z1) * (x3 - x1) - (x2 - x1) * (z3 - z1);
        float nz = (x2 - x1) * (y3 - y1) - (y2 - y1) * (x3 - x1);
        float length = sqrtf(nx * nx + ny * ny + nz * nz);
        float* h = helpers + (size_t)t * 12;
        h[0] = nx / length; h[1] = ny / length; h[2] = nz / length;
        h[3] = x3 - x1; h[4] = y3 - y1; h[5] = z3 - z1;
        h[6] = x2 - x1; h[7] = y2 - y1; h[8] = z2 - z1;
        h[9] = (x3 - x1) * (x2 - x1) + (y3 - y1) * (y2 - y1) + (z3 - z1) * (z2 - z1);
        h[10] = (x3 - x1) * (x3 - x1) + (y3 - y1) * (y3 - y1) + (z3 - z1) * (z3 - z1);
        h[11] = (x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1) + (z2 - z1) * (z2 - z1);
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* calcCubePos / calcCubeHash: dSim3/src/spinSystem.cpp:691-721, 756-759     */
/* std::max(0.0f, std::min(floor((p+1)/L), n-1)) then cast to uint           */
/* ------------------------------------------------------------------------ */
static inline uint32_t cube_coord(float p, float L, uint32_t n) {
    float f = floorf((p + 1.0f) / L);
    float hi = (float)(n - 1);
    float mn = (hi < f) ? hi : f;          /* std::min(f, hi)  */
    float mx = (0.0f < mn) ? mn : 0.0f;    /* std::max(0, mn)  */
    return (uint32_t)mx;
}

/* ------------------------------------------------------------------------ */
/* populateCubes helpers: pointInCube :1355-1357, rayTriangleIntersect :1360 */
/* ------------------------------------------------------------------------ */
static inline float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline f3 sub3(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }

static int point_in_cube(f3 p, f3 mn, f3 mx) {
    return ((p.x <= mx.x) && (p.x >= mn.x)) && ((p.y <= mx.y) && (p.y >= mn.y)) &&
           ((p.z <= mx.z) && (p.z >= mn.z));
}
static int ray_tri(f3 rp1, f3 rp2, f3 tp1, f3 tp2, f3 tp3) {
    f3 u = sub3(tp2, tp1);
    f3 v = sub3(tp3, tp1);
    f3 n = mk(u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x);
    float nlength = sqrtf(n.x * n.x + n.y * n.y + n.z * n.z);
    float s = 2.0f, t = 2.0f;
    n.x = n.x / nlength; n.y = n.y / nlength; n.z = n.z / nlength;
    float r = dot3(n, sub3(tp1, rp1)) / dot3(n, sub3(rp2, rp1));
    if ((0 < r) & (r < 1)) {
        f3 d = sub3(rp2, rp1);
        f3 w = sub3(mk(rp1.x + d.x * r, rp1.y + d.y * r, rp1.z + d.z * r), tp1);
        s = (dot3(u, v) * dot3(w, v) - dot3(v, v) * dot3(w, u)) /
            (dot3(u, v) * dot3(u, v) - dot3(u, u) * dot3(v, v));
        t = (dot3(u, v) * dot3(w, u) - dot3(u, u) * dot3(w, v)) /
            (dot3(u, v) * dot3(u, v) - dot3(u, u) * dot3(v, v));
    }
    return (s >= 0) && (t >= 0) && (s + t <= 1);
}

/* Cube corner with bit 0 = x max, bit 1 = y max, bit 2 = z max. */
static inline f3 corner(f3 mn, f3 mx, int b) {
    return mk((b & 1) ? mx.x : mn.x, (b & 2) ? mx.y : mn.y, (b & 4) ? mx.z : mn.z);
}
/* The 12 cube edges (start, end) and 12 face triangles, in the argument
 * order of spinSystem.cpp:1192-1203 and :1208-1219. */
static const unsigned char k_edges[12][2] = {
    {0, 1}, {0, 2}, {0, 4}, {6, 2}, {6, 4}, {6, 7},
    {3, 2}, {3, 1}, {3, 7}, {5, 7}, {5, 1}, {5, 4}};
static const unsigned char k_faces[12][3] = {
    {0, 1, 2}, {0, 4, 2}, {0, 4, 1}, {6, 2, 4}, {6, 2, 7}, {6, 4, 7},
    {3, 2, 1}, {3, 7, 1}, {3, 7, 2}, {5, 4, 7}, {5, 1, 7}, {5, 4, 1}};

static int tri_cube_overlap(f3 p1, f3 p2, f3 p3, f3 cmin, f3 cmax) {
    if (point_in_cube(p1, cmin, cmax) || point_in_cube(p2, cmin, cmax) ||
        point_in_cube(p3, cmin, cmax))
        return 1;
    for (int e = 0; e < 12; e++)
        if (ray_tri(corner(cmin, cmax, k_edges[e][0]), corner(cmin, cmax, k_edges[e][1]), p1, p2, p3))
            return 1;
    const f3 a[3] = {p1, p1, p2}, b[3] = {p2, p3, p3};
    for (int k = 0; k < 3; k++)
        for (int f = 0; f < 12; f++)
            if (ray_tri(a[k], b[k], corner(cmin, cmax, k_faces[f][0]),
                        corner(cmin, cmax, k_faces[f][1]), corner(cmin, cmax, k_faces[f][2])))
                return 1;
    return 0;
}

static void populate(uint32_t nT, const float* V, const uint32_t* trgls, uint32_t n,
                     uint32_t maxTPC, uint32_t* counter, uint32_t* list, uint32_t* maxOut) {
    float L = 2.0f / (float)n;  /* m_cubeLength = 2.0f / m_numCubes, :1115 */
    size_t total = (size_t)n * n * n;
    memset(counter, 0, total * sizeof(uint32_t));
    uint32_t maxc = 0;
    for (uint32_t t = 0; t < nT; t++) {
        uint32_t i1 = trgls[t * 3], i2 = trgls[t * 3 + 1], i3 = trgls[t * 3 + 2];
        f3 p1 = mk(V[i1 * 3], V[i1 * 3 + 1], V[i1 * 3 + 2]);
        f3 p2 = mk(V[i2 * 3], V[i2 * 3 + 1], V[i2 * 3 + 2]);
        f3 p3 = mk(V[i3 * 3], V[i3 * 3 + 1], V[i3 * 3 + 2]);
        f3 mn = p1, mx = p1;
        if (p2.x < mn.x) mn.x = p2.x; if (p3.x < mn.x) mn.x = p3.x;
        if (p2.y < mn.y) mn.y = p2.y; if (p3.y < mn.y) mn.y = p3.y;
        if (p2.z < mn.z) mn.z = p2.z; if (p3.z < mn.z) mn.z = p3.z;
        if (p2.x > mx.x) mx.x = p2.x; if (p3.x > mx.x) mx.x = p3.x;
        if (p2.y > mx.y) mx.y = p2.y; if (p3.y > mx.y) mx.y = p3.y;
        if (p2.z > mx.z) mx.z = p2.z; if (p3.z > mx.z) mx.z = p3.z;
        uint32_t x0 = cube_coord(mn.x, L, n), y0 = cube_coord(mn.y, L, n), z0 = cube_coord(mn.z, L, n);
        uint32_t x1 = cube_coord(mx.x, L, n), y1 = cube_coord(mx.y, L, n), z1 = cube_coord(mx.z, L, n);
        for (uint32_t xc = x0; xc <= x1; xc++)
            for (uint32_t yc = y0; yc <= y1; yc++)
                for (uint32_t zc = z0; zc <= z1; zc++) {
                    uint32_t cube = n * n * zc + n * yc + xc;
                    f3 cmin = mk(-1 + xc * L, -1 + yc * L, -1 + zc * L);
                    f3 cmax = mk(-1 + (xc + 1) * L, -1 + (yc + 1) * L, -1 + (zc + 1) * L);
                    if (tri_cube_overlap(p1, p2, p3, cmin, cmax)) {
                        if (list) list[(size_t)cube * maxTPC + counter[cube]] = t;
                        counter[cube]++;
                        if (counter[cube] > maxc) maxc = counter[cube];
                    }
                }
    }
    if (maxOut) *maxOut = maxc;
}

uint32_t or3_populate_count(uint32_t nT, const float* vertices, const uint32_t* trgls,
                            uint32_t numCubes, uint32_t* cubeCounter) {
    uint32_t m = 0;
    populate(nT, vertices, trgls, numCubes, 0, cubeCounter, NULL, &m);
    return m;
}
void or3_populate_fill(uint32_t nT, const float* vertices, const uint32_t* trgls,
                       uint32_t numCubes, uint32_t maxTPC, uint32_t* cubeCounter,
                       uint32_t* trianglesInCubes) {
    populate(nT, vertices, trgls, numCubes, maxTPC, cubeCounter, trianglesInCubes, NULL);
}

/* ------------------------------------------------------------------------ */
/* The step.  FP32 instantiation restates spinKernelCpu.cpp exactly; the    */
/* FP64 instantiation is the same algorithm in double (precision oracle).   */
/* ------------------------------------------------------------------------ */
#define REAL float
#define SFX(name) name##_f32
#define RLIT(x) x##f
#include "dsim3_step.inc"
#undef REAL
#undef SFX
#undef RLIT

#define REAL double
#define SFX(name) name##_f64
#define RLIT(x) x
#include "dsim3_step.inc"
#undef REAL
#undef SFX
#undef RLIT

uint32_t or3_integrate(const or3_params* p, uint32_t N, float* pos, uint32_t* seed,
                       float* mag, float* phase, uint8_t* comp, uint16_t* fiber,
                       const float* vertices, const float* helpers,
                       const uint32_t* triInfo, const uint32_t* cubeCounter,
                       const uint32_t* trianglesInCubes, float gx, float gy, float gz,
                       float phaseConstant, uint32_t iterations, const float* draws,
                       float* drawsOut, uint32_t* counts) {
    uint32_t capped = 0;
    /* updateSpins CPU branch, spinSystem.cpp:1964-1968: iterations x all spins */
    for (uint32_t it = 0; it < iterations; it++) {
        for (uint32_t i = 0; i < N; i++) {
            float d[4];
            if (draws) {
                const float* src = draws + ((size_t)it * N + i) * 4;
                d[0] = src[0]; d[1] = src[1]; d[2] = src[2]; d[3] = src[3];
            } else {
                or_myrandn(seed + 2 * (size_t)i, d);
            }
            if (drawsOut) memcpy(drawsOut + ((size_t)it * N + i) * 4, d, sizeof(d));
            capped += step_f32(p, pos + 3 * (size_t)i, mag + i, phase + i, comp + i, fiber + i,
                               vertices, helpers, triInfo, cubeCounter, trianglesInCubes,
                               gx, gy, gz, phaseConstant, d, counts ? counts + 2 * (size_t)i : NULL);
        }
    }
    return capped;
}

/* The same loop with the spin loop of each iteration spread over threads, as
 * the reference's OpenMP patch does (dSim3/parallelization_cpu.diff:38);
 * MWC draws only (each spin owns its seeds).  Used to time the CPU path. */
uint32_t or3_integrate_mt(const or3_params* p, uint32_t N, float* pos, uint32_t* seed,
                          float* mag, float* phase, uint8_t* comp, uint16_t* fiber,
                          const float* vertices, const float* helpers,
                          const uint32_t* triInfo, const uint32_t* cubeCounter,
                          const uint32_t* trianglesInCubes, float gx, float gy, float gz,
                          float phaseConstant, uint32_t iterations, int nthreads) {
    uint32_t capped = 0;
    for (uint32_t it = 0; it < iterations; it++) {
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads) reduction(+ : capped)
        for (uint32_t i = 0; i < N; i++) {
            float d[4];
            or_myrandn(seed + 2 * (size_t)i, d);
            capped += step_f32(p, pos + 3 * (size_t)i, mag + i, phase + i, comp + i, fiber + i,
                               vertices, helpers, triInfo, cubeCounter, trianglesInCubes,
                               gx, gy, gz, phaseConstant, d, NULL);
        }
    }
    return capped;
}

uint32_t or3_integrate_multi(const or3_params* p, uint32_t N, float* pos, uint32_t* seed,
                             float* mag, uint8_t* comp, uint16_t* fiber,
                             const float* vertices, const float* helpers,
                             const uint32_t* triInfo, const uint32_t* cubeCounter,
                             const uint32_t* trianglesInCubes, uint32_t nG, const float* grads,
                             const float* wave, float phaseConstant, uint32_t iterations,
                             const float* draws, float* phases, uint32_t* counts, int nthreads) {
    uint32_t capped = 0;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads) reduction(+ : capped)
    for (uint32_t i = 0; i < N; i++) {
        float* q = pos + 3 * (size_t)i;
        float* ph = phases + (size_t)i * nG;
        for (uint32_t it = 0; it < iterations; it++) {
            float d[4];
            if (draws) {
                const float* src = draws + ((size_t)it * N + i) * 4;
                d[0] = src[0]; d[1] = src[1]; d[2] = src[2]; d[3] = src[3];
            } else {
                or_myrandn(seed + 2 * (size_t)i, d);
            }
            float unused = 0.0f;
            capped += step_f32(p, q, mag + i, &unused, comp + i, fiber + i, vertices, helpers, triInfo,
                               cubeCounter, trianglesInCubes, 0.0f, 0.0f, 0.0f, phaseConstant, d,
                               counts ? counts + 2 * (size_t)i : NULL);
            const float w = wave[it];
            for (uint32_t k = 0; k < nG; k++) {
                float gx = w * grads[3 * k], gy = w * grads[3 * k + 1], gz = w * grads[3 * k + 2];
                ph[k] += (gx * q[0] + gy * q[1] + gz * q[2]) * phaseConstant;
            }
        }
    }
    return capped;
}

uint32_t or3_integrate_f64(const or3_params* p, uint32_t N, double* pos, double* mag,
                           double* phase, uint8_t* comp, uint16_t* fiber,
                           uint32_t nT, const double* vertices, const uint32_t* trgls,
                           const uint32_t* triInfo, const uint32_t* cubeCounter,
                           const uint32_t* trianglesInCubes, const double* gradPerStep,
                           double phaseConstant, uint32_t iterations, const float* draws,
                           uint32_t* counts) {
    /* helpers in double, same formulas as spinSystem.cpp:612-648 */
    double* H = (double*)malloc((size_t)nT * 12 * sizeof(double));
    if (!H) return 0xFFFFFFFFu;
    for (uint32_t t = 0; t < nT; t++) {
        const double* a = vertices + 3 * (size_t)trgls[t * 3];
        const double* b = vertices + 3 * (size_t)trgls[t * 3 + 1];
        const double* c = vertices + 3 * (size_t)trgls[t * 3 + 2];
        double nx = (b[1] - a[1]) * (c[2] - a[2]) - (b[2] - a[2]) * (c[1] - a[1]);
        double ny = (b[2] - a[2]) * (c[0] - a[0]) - (b[0] - a[0]) * (c[2] - a[2]);
        double nz = (b[0] - a[0]) * (c[1] - a[1]) - (b[1] - a[1]) * (c[0] - a[0]);
        double len = sqrt(nx * nx + ny * ny + nz * nz);
        double* h = H + (size_t)t * 12;
        h[0] = nx / len; h[1] = ny / len; h[2] = nz / len;
        h[3] = c[0] - a[0]; h[4] = c[1] - a[1]; h[5] = c[2] - a[2];
        h[6] = b[0] - a[0]; h[7] = b[1] - a[1]; h[8] = b[2] - a[2];
        h[9] = h[3] * h[6] + h[4] * h[7] + h[5] * h[8];
        h[10] = h[3] * h[3] + h[4] * h[4] + h[5] * h[5];
        h[11] = h[6] * h[6] + h[7] * h[7] + h[8] * h[8];
    }
    uint32_t capped = 0;
    for (uint32_t it = 0; it < iterations; it++) {
        double gx = gradPerStep[3 * (size_t)it], gy = gradPerStep[3 * (size_t)it + 1],
               gz = gradPerStep[3 * (size_t)it + 2];
        for (uint32_t i = 0; i < N; i++) {
            const float* src = draws + ((size_t)it * N + i) * 4;
            double d[4] = {src[0], src[1], src[2], src[3]};
            capped += step_f64(p, pos + 3 * (size_t)i, mag + i, phase + i, comp + i, fiber + i,
                               vertices, H, triInfo, cubeCounter, trianglesInCubes,
                               gx, gy, gz, phaseConstant, d, counts ? counts + 2 * (size_t)i : NULL);
        }
    }
    free(H);
    return capped;
}

/* FP64 walk that records gradient moments instead of one phase: for every
 * waveform k (waves[k * iterations + t]) M_k += w_k(t) * pos(t) after each
 * step, in double.  The phase of a gradient g with waveform k is then
 * phaseConstant * (g . M_k), the quantity the GPU batch form accumulates.
 * Spins are independent, so they run in parallel (OpenMP); counts may be NULL. */
uint32_t or3_integrate_f64_moments(const or3_params* p, uint32_t N, double* pos, double* mag,
                                   uint8_t* comp, uint16_t* fiber, uint32_t nT,
                                   const double* vertices, const uint32_t* trgls,
                                   const uint32_t* triInfo, const uint32_t* cubeCounter,
                                   const uint32_t* trianglesInCubes, uint32_t nWaves,
                                   const double* waves, uint32_t iterations, const float* draws,
                                   double* moments, uint32_t* counts, int nthreads) {
    double* H = (double*)malloc((size_t)nT * 12 * sizeof(double));
    if (!H) return 0xFFFFFFFFu;
    for (uint32_t t = 0; t < nT; t++) {
        const double* a = vertices + 3 * (size_t)trgls[t * 3];
        const double* b = vertices + 3 * (size_t)trgls[t * 3 + 1];
        const double* c = vertices + 3 * (size_t)trgls[t * 3 + 2];
        double nx = (b[1] - a[1]) * (c[2] - a[2]) - (b[2] - a[2]) * (c[1] - a[1]);
        double ny = (b[2] - a[2]) * (c[0] - a[0]) - (b[0] - a[0]) * (c[2] - a[2]);
        double nz = (b[0] - a[0]) * (c[1] - a[1]) - (b[1] - a[1]) * (c[0] - a[0]);
        double len = sqrt(nx * nx + ny * ny + nz * nz);
        double* h = H + (size_t)t * 12;
        h[0] = nx / len; h[1] = ny / len; h[2] = nz / len;
        h[3] = c[0] - a[0]; h[4] = c[1] - a[1]; h[5] = c[2] - a[2];
        h[6] = b[0] - a[0]; h[7] = b[1] - a[1]; h[8] = b[2] - a[2];
        h[9] = h[3] * h[6] + h[4] * h[7] + h[5] * h[8];
        h[10] = h[3] * h[3] + h[4] * h[4] + h[5] * h[5];
        h[11] = h[6] * h[6] + h[7] * h[7] + h[8] * h[8];
    }
    uint32_t capped = 0;
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads) reduction(+ : capped)
    for (int64_t ii = 0; ii < (int64_t)N; ii++) {
        const uint32_t i = (uint32_t)ii;
        double phase = 0.0;
        double* M = moments + (size_t)i * nWaves * 3;
        for (uint32_t it = 0; it < iterations; it++) {
            const float* src = draws + ((size_t)it * N + i) * 4;
            double d[4] = {src[0], src[1], src[2], src[3]};
            capped += step_f64(p, pos + 3 * (size_t)i, mag + i, &phase, comp + i, fiber + i, vertices, H,
                               triInfo, cubeCounter, trianglesInCubes, 0.0, 0.0, 0.0, 0.0, d,
                               counts ? counts + 2 * (size_t)i : NULL);
            const double* P = pos + 3 * (size_t)i;
            for (uint32_t k = 0; k < nWaves; k++) {
                const double w = waves[(size_t)k * iterations + it];
                M[3 * k] += w * P[0];
                M[3 * k + 1] += w * P[1];
                M[3 * k + 2] += w * P[2];
            }
        }
    }
    free(H);
    return capped;
}

/* getMrSignal(double mrSignal[]), spinSystem.cpp:1452-1500 */
void or3_signal(uint32_t N, const float* mag, const float* phase, const uint8_t* comp,
                double out[5]) {
    double X[5] = {0}, Y[5] = {0};
    uint32_t n[5] = {0};
    for (uint32_t i = 0; i < N; i++) {
        uint32_t c = comp[i];
        /* cos/sin of a float resolve to the float overloads in the reference's
         * C++ build, so each term is a float product widened to double. */
        X[0] += (double)(cosf(phase[i]) * mag[i]);
        Y[0] += (double)(sinf(phase[i]) * mag[i]);
        n[0]++;
        X[c + 1] += (double)(cosf(phase[i]) * mag[i]);
        Y[c + 1] += (double)(sinf(phase[i]) * mag[i]);
        n[c + 1]++;
    }
    for (int c = 0; c < 5; c++)
        out[c] = n[c] == 0 ? 0.0 : sqrt(X[c] * X[c] + Y[c] * Y[c]) / (double)n[c];
}
