// compartments.cu -- which compartment and fiber each spin starts in (GPU).
//
// Reference: SpinSystem::findSpinsInFibers, dSim3/src/spinSystem.cpp:1615-1852.
// A line is drawn from the spin out of the volume along the axis of its
// largest coordinate, to 1.1 times the mesh extent on that axis
// (spinSystem.cpp:1676-1684).  A closed membrane encloses the spin when the
// line crosses it an odd number of times; membranes are examined innermost
// type first (axon 0, myelin 1, glia 2), giving compartment 1, 2 or 3, else 0
// (outside).  If the line touches a triangle edge or vertex the answer is
// ambiguous and the line is tilted by a random offset of up to 0.05 per axis
// and tried again (:1686-1692); after 20 failed tries the spin is moved to a
// random position and examined anew (:1659-1665).
//
// Here one thread follows one spin's line through the fine acceleration grid:
// every cell of the line's bounding box is scanned, and a crossing is counted
// only in the cell that contains the crossing point, so a triangle listed in
// several cells counts once.  Crossing parity is kept per (fiber, membrane).
// The reference takes its candidates from an R-tree in tree order; when two
// fibers of the same membrane type both enclose a spin (overlapping meshes)
// it keeps the last one in that order, while this kernel keeps the lowest
// fiber index.  For meshes without overlaps the result is the same.
// Tilts and moves draw from Philox keyed by the caller's seed and the spin.
#include "common.cuh"
#include "engine.h"
#include "mesh_common.cuh"

namespace dsim {

static constexpr int kParitySlots = 32;

__device__ __forceinline__ float sgn_ref(float v) { return (v >= 0.0f) ? 1.0f : -1.0f; }

__global__ void __launch_bounds__(128) k_compartments(MeshDev g, AccelDev acc, SpinsSorted S, float mx, float my,
                                                      float mz, float startBox, uint32_t key0, uint32_t key1,
                                                      uint32_t maxTries, uint32_t maxMoves, uint32_t* status,
                                                      uint32_t* moved) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.N) return;
    float sx = S.x[i], sy = S.y[i], sz = S.z[i];
    const uint32_t id = S.id[i];
    uint32_t keys[kParitySlots];
    uint32_t parity = 0, nkeys = 0;
    bool resolved = false;
    uint32_t comp = 0, fiber = 0xFFFFu, st = 0, nMoves = 0;
    for (uint32_t move = 0; move <= maxMoves && !resolved; move++) {
        if (move > 0) {
            // spinSystem.cpp:1659-1665: a new random position in the start box
            const u32x4 r = philox4x32_10({id, move, 0u, 0xB0C5u}, key0, key1);
            sx = startBox * 2.0f * ((float)(r.x >> 8) * 0x1p-24f - 0.5f);
            sy = startBox * 2.0f * ((float)(r.y >> 8) * 0x1p-24f - 0.5f);
            sz = startBox * 2.0f * ((float)(r.z >> 8) * 0x1p-24f - 0.5f);
            nMoves++;
        }
        for (uint32_t tr = 0; tr <= maxTries && !resolved; tr++) {
            float ex = sx, ey = sy, ez = sz;
            const float ax = fabsf(sx), ay = fabsf(sy), az = fabsf(sz);
            if ((ax > ay) & (ax > az)) ex = (float)((double)sgn_ref(sx) * 1.1 * (double)mx);
            else if (ay > az) ey = (float)((double)sgn_ref(sy) * 1.1 * (double)my);
            else ez = (float)((double)sgn_ref(sz) * 1.1 * (double)mz);
            if (tr > 0) {
                const u32x4 r = philox4x32_10({id, tr, move, 0xC0A5u}, key0, key1);
                ex = (float)((double)ex + (double)((float)(r.x >> 8) * 0x1p-24f) * 0.05);
                ey = (float)((double)ey + (double)((float)(r.y >> 8) * 0x1p-24f) * 0.05);
                ez = (float)((double)ez + (double)((float)(r.z >> 8) * 0x1p-24f) * 0.05);
            }
            const float dx = ex - sx, dy = ey - sy, dz = ez - sz;
            const uint32_t lo0 = fine_coord(fminf(sx, ex) - kAccelEps, acc.invLf, acc.nf);
            const uint32_t lo1 = fine_coord(fminf(sy, ey) - kAccelEps, acc.invLf, acc.nf);
            const uint32_t lo2 = fine_coord(fminf(sz, ez) - kAccelEps, acc.invLf, acc.nf);
            const uint32_t hi0 = fine_coord(fmaxf(sx, ex) + kAccelEps, acc.invLf, acc.nf);
            const uint32_t hi1 = fine_coord(fmaxf(sy, ey) + kAccelEps, acc.invLf, acc.nf);
            const uint32_t hi2 = fine_coord(fmaxf(sz, ez) + kAccelEps, acc.invLf, acc.nf);
            nkeys = 0;
            parity = 0;
            uint32_t edgeTypes = 0;  // membrane types whose triangles were met at an edge or vertex
            for (uint32_t c2 = lo2; c2 <= hi2; c2++)
                for (uint32_t c1 = lo1; c1 <= hi1; c1++)
                    for (uint32_t c0 = lo0; c0 <= hi0; c0++) {
                        const uint32_t key = morton3(c0, c1, c2);
                        const uint32_t b0 = __ldg(acc.start + key), b1 = __ldg(acc.start + key + 1);
                        for (uint32_t k = b0; k < b1; k++) {
                            FastHit h;
                            if (!test_entry(g, acc, k, 0xFFFFFFFFu, sx, sy, sz, dx, dy, dz, h)) continue;
                            const uint32_t t = h.t;
                            // count the crossing in the cell that holds it
                            if (fine_coord(h.x, acc.invLf, acc.nf) != c0 || fine_coord(h.y, acc.invLf, acc.nf) != c1 ||
                                fine_coord(h.z, acc.invLf, acc.nf) != c2)
                                continue;
                            const uint32_t info = __ldg(&g.plane[t].info);
                            if (h.type > 1) edgeTypes |= 1u << (info & 3u);
                            const uint32_t fk = info;  // fiber << 2 | membrane
                            uint32_t s = 0;
                            while (s < nkeys && keys[s] != fk) s++;
                            if (s == nkeys) {
                                if (nkeys == kParitySlots) { st |= kStatusParityOverflow; continue; }
                                keys[nkeys++] = fk;
                            }
                            parity ^= 1u << s;
                        }
                    }
            uint32_t c = 0, f = 0xFFFFu, mt = 0;
            for (; mt < 3 && c == 0; mt++) {
                uint32_t best = 0xFFFFFFFFu;
                for (uint32_t s = 0; s < nkeys; s++)
                    if (((parity >> s) & 1u) && (keys[s] & 3u) == mt && (keys[s] >> 2) < best) best = keys[s] >> 2;
                if (best != 0xFFFFFFFFu) {
                    c = (mt == 0) ? 1u : ((mt == 2) ? 3u : 2u);
                    f = best & 0xFFFFu;
                }
            }
            // the membrane types examined (up to the one that encloses the spin)
            // must be free of edge and vertex crossings, as in the reference
            if (edgeTypes & ((1u << mt) - 1u)) continue;  // ambiguous: tilt the line and try again
            resolved = true;
            comp = c;
            fiber = f;
        }
    }
    if (!resolved) st |= kStatusUnresolved;
    S.x[i] = sx; S.y[i] = sy; S.z[i] = sz;
    S.meta[i] = (comp & 0xFFu) | (fiber << 8);
    if (nMoves) atomicAdd(moved, nMoves);
    if (st) atomicOr(status, st);
}

int launch_compartments(const MeshDev& g, const AccelDev& acc, const SpinsSorted& S, const float maxabs[3],
                        float startBox, uint64_t seed, uint32_t maxTries, uint32_t maxMoves, uint32_t* status,
                        uint32_t* moved, cudaStream_t st) {
    if (S.N == 0) return kOk;
    k_compartments<<<(S.N + 127) / 128, 128, 0, st>>>(g, acc, S, maxabs[0], maxabs[1], maxabs[2], startBox,
                                                      (uint32_t)seed, (uint32_t)(seed >> 32), maxTries, maxMoves,
                                                      status, moved);
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}

}  // namespace dsim
