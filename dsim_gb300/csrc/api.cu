// api.cu -- host side of the native engine: substrate loading and grid build,
// device-resident spin state, launches, and the dsim_* C-ABI (include/dsim.h).
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <limits>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#pragma GCC visibility push(default)
#include "../../include/dsim.h"
#pragma GCC visibility pop
#include "common.cuh"
#include "engine.h"
#include "host_formats.h"

namespace dsim {

static thread_local std::string g_last_error;

void set_last_error(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = std::string("dsim error ") + std::to_string(code) + ": " + buf;
}
void set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line) {
    set_last_error(kErrCuda, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
}
const char* last_error_message() { return g_last_error.c_str(); }

template <typename T>
static int dev_alloc(T** p, size_t count, uint64_t* bytes = nullptr) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
    if (e != cudaSuccess) {
        set_last_error(kErrNoMem, "cudaMalloc(%zu bytes): %s", count * sizeof(T), cudaGetErrorString(e));
        cudaGetLastError();
        return kErrNoMem;
    }
    if (bytes) *bytes += count * sizeof(T);
    return kOk;
}

}  // namespace dsim

using namespace dsim;

struct dsim_mesh {
    uint32_t nV = 0, nT = 0, nFibers = 0, n = 50;
    float L = 0.04f;
    uint64_t entries = 0, maxPerCell = 0, nonempty = 0, bytes = 0;
    float* V = nullptr;
    uint32_t* trgls = nullptr;
    uint32_t* membrane = nullptr;
    uint32_t* fiber = nullptr;
    TriPlane* plane = nullptr;
    TriBary* bary = nullptr;
    uint32_t* cell_start = nullptr;
    uint32_t* cell_tri = nullptr;
    Tri64* tri64 = nullptr;  // FP64 helpers, built for the first precision-form job
    uint4* tri_cells = nullptr;  // each triangle's reference cells (up to 4)
    // fine acceleration grid (nf = 0: none; steps scan the reference grid)
    uint32_t nf = 0;
    uint32_t kernel = 8;  // 5/6/7 warp-flattened (8, 6, 4 blocks per SM), 8 with the plane-survivor queue, 9 TMA staging
                          // (8, 6, 4), 8 flattened with queued plane survivors, 9 with staged records
    uint64_t accEntries = 0, accBytes = 0;
    uint32_t* acc_start = nullptr;
    AccelRec* acc_rec = nullptr;
    uint32_t* acc_tri = nullptr;
    AccelRecWide* acc_recw = nullptr;
    AccelRecFull* acc_recf = nullptr;
    uint32_t accWide = 1;  // fine-grid records: 0 16-byte, 1 32-byte, 2 64-byte
    float maxabs[3] = {1.0f, 1.0f, 1.0f};  // max(1, max |vertex coordinate|) per axis, as initFibers keeps
    MeshDev dev() const {
        MeshDev g;
        g.cell_start = cell_start; g.cell_tri = cell_tri; g.plane = plane; g.bary = bary;
        g.tri64 = tri64;
        g.tri_cells = tri_cells;
        g.n = n; g.L = L;
        return g;
    }
    AccelDev acc() const {
        AccelDev a;
        a.start = acc_start; a.rec = acc_rec; a.tri = acc_tri; a.recw = acc_recw; a.recf = acc_recf; a.nf = nf;
        a.invLf = (float)nf / 2.0f; a.wide = acc_recf ? 2u : (acc_recw ? 1u : 0u);
        return a;
    }
};

// (Re)build the fine acceleration grid with nf cells per axis (0 removes it).
static int accel_build(dsim_mesh* m, uint32_t nf) {
    cudaFree(m->acc_start); cudaFree(m->acc_rec); cudaFree(m->acc_tri); cudaFree(m->acc_recw); cudaFree(m->acc_recf);
    m->acc_start = nullptr; m->acc_rec = nullptr; m->acc_tri = nullptr; m->acc_recw = nullptr; m->acc_recf = nullptr;
    m->nf = 0; m->accEntries = 0; m->accBytes = 0;
    if (nf == 0) return kOk;
    if (nf > 1024) { set_last_error(kErrTooLarge, "accel grid: %u cells per axis > 1024", nf); return kErrTooLarge; }
    uint32_t nkeys = accel_keys(nf);
    int rc;
    uint32_t* counter = nullptr;
    uint32_t* scratch = nullptr;
    cudaStream_t st = 0;
    if ((rc = dev_alloc(&counter, nkeys))) return rc;
    if ((rc = dev_alloc(&scratch, scan_scratch_words(nkeys)))) { cudaFree(counter); return rc; }
    do {
        if ((rc = dev_alloc(&m->acc_start, (size_t)nkeys + 1, &m->accBytes))) break;
        if (cudaMemsetAsync(counter, 0, (size_t)nkeys * 4, st) != cudaSuccess) { rc = kErrCuda; break; }
        if ((rc = launch_accel_cells(false, m->nT, m->plane, m->bary, nf, counter, nullptr, nullptr, nullptr, nullptr, st))) break;
        if ((rc = launch_scan_exclusive(counter, m->acc_start, nkeys, scratch, st))) break;
        uint32_t total = 0;
        if (cudaMemcpyAsync(&total, m->acc_start + nkeys, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) { rc = kErrCuda; break; }
        m->accEntries = total;
        if (m->accWide == 2) {
            if ((rc = dev_alloc(&m->acc_recf, total, &m->accBytes))) break;
        } else if (m->accWide) {
            if ((rc = dev_alloc(&m->acc_recw, total, &m->accBytes))) break;
        } else {
            if ((rc = dev_alloc(&m->acc_rec, total, &m->accBytes))) break;
            if ((rc = dev_alloc(&m->acc_tri, total, &m->accBytes))) break;
        }
        if (cudaMemsetAsync(counter, 0, (size_t)nkeys * 4, st) != cudaSuccess) { rc = kErrCuda; break; }
        if ((rc = launch_accel_cells(true, m->nT, m->plane, m->bary, nf, counter, m->acc_start, m->acc_rec, m->acc_tri, m->acc_recw, st, m->acc_recf))) break;
        if (cudaStreamSynchronize(st) != cudaSuccess) { rc = kErrCuda; break; }
        m->nf = nf;
    } while (0);
    if (rc == kErrCuda) set_last_error(kErrCuda, "accel grid build: %s", cudaGetErrorString(cudaGetLastError()));
    cudaFree(counter);
    cudaFree(scratch);
    if (rc) {
        cudaFree(m->acc_start); cudaFree(m->acc_rec); cudaFree(m->acc_tri); cudaFree(m->acc_recw); cudaFree(m->acc_recf);
        m->acc_start = nullptr; m->acc_rec = nullptr; m->acc_tri = nullptr; m->acc_recw = nullptr; m->acc_recf = nullptr; m->nf = 0;
    }
    return rc;
}

struct dsim_cyl {
    CylHost host;
    float4* fibers = nullptr;
    uint32_t* cc = nullptr;
    uint32_t* cubes = nullptr;
    float4* cubeF = nullptr;  // each grid entry's fiber record
    uint32_t* fineStart = nullptr;  // fine filter grid (CSR), null when not built
    float4* fineRec = nullptr;
    uint32_t* finePos = nullptr;
    uint32_t fineK = 0;
    uint64_t fineEntries = 0, fineBytes = 0;
    uint64_t bytes = 0;
    CylDev dev() const {
        CylDev g;
        g.fibers = fibers; g.cube_count = cc; g.cubes = cubes; g.cube_fibers = cubeF;
        g.n = host.numCubes; g.maxFPC = host.maxFPC; g.L = host.cubeLength;
        g.nF = host.nF;
        g.fine_start = fineK ? fineStart : nullptr; g.fine_rec = fineRec; g.fine_pos = finePos;
        g.fineK = fineK;
        g.fineInv = fineK ? (float)fineK / host.cubeLength : 0.0f;
        return g;
    }
};

// batches holding each cylinder substrate's device view: its fine grid is
// not rebuilt (freed) while one does
static std::mutex g_cylHoldMu;
static std::unordered_map<const dsim_cyl*, int> g_cylHolds;

namespace dsim {
// device views for the batch module (batch.cu)
int mesh_views(const dsim_mesh* m, MeshDev* g, AccelDev* a) {
    if (!m || !g || !a) return kErrInvalid;
    if (m->nf == 0 || !(m->acc_recw || m->acc_recf)) {
        set_last_error(kErrInvalid, "batch: the mesh needs its fine grid with 32- or 64-byte records");
        return kErrInvalid;
    }
    *g = m->dev();
    *a = m->acc();
    return kOk;
}
int mesh_tri64(dsim_mesh* m) {
    if (!m) return kErrInvalid;
    // batches on several host threads may share the mesh: one builds the table
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    if (m->tri64 || m->nT == 0) return kOk;
    Tri64* t = nullptr;
    int rc = dev_alloc(&t, m->nT, &m->bytes);
    if (rc) return rc;
    if ((rc = launch_tri64(m->nT, m->V, m->trgls, t, 0))) { cudaFree(t); return rc; }
    DSIM_CUDA_TRY(cudaDeviceSynchronize());
    m->tri64 = t;
    return kOk;
}
int cyl_view(const dsim_cyl* c, CylDev* g) {
    if (!c || !g) return kErrInvalid;
    *g = c->dev();
    return kOk;
}
void cyl_hold(const dsim_cyl* c, int delta) {
    std::lock_guard<std::mutex> lk(g_cylHoldMu);
    if (delta > 0) {
        g_cylHolds[c] += delta;
    } else {
        auto it = g_cylHolds.find(c);
        if (it != g_cylHolds.end() && (it->second += delta) <= 0) g_cylHolds.erase(it);
    }
}
int mesh_rebuild_accel(dsim_mesh* m, uint32_t nf) { return accel_build(m, nf); }
}  // namespace dsim

struct dsim_spins {
    uint32_t N = 0;
    cudaStream_t st = nullptr;
    float *x = nullptr, *y = nullptr, *z = nullptr, *mag = nullptr, *phase = nullptr;
    uint32_t* meta = nullptr;
    // reordering by cell (fast mesh path): stable ids, second buffer set
    uint32_t* id = nullptr;
    float *x2 = nullptr, *y2 = nullptr, *z2 = nullptr, *mag2 = nullptr, *phase2 = nullptr;
    uint32_t *meta2 = nullptr, *id2 = nullptr, *keys = nullptr, *hist = nullptr, *hstart = nullptr,
             *hscratch = nullptr;
    uint32_t sortNb = 0;        // key grid of the allocated sort buffers
    uint32_t sortEvery = 1000;  // steps between reorderings (0 = never): once per call of up to 1000 steps
    uint64_t launches = 0;      // kernels launched by dsim_mesh_run / dsim_cyl_run on this object
    uint32_t spinBase = 0;      // global index of spin 0 in the Philox counter (replica shards)
    bool permuted = false;      // slot i does not hold spin i
    float4* cpos = nullptr;     // cylinder layout (lazy)
    uint32_t* cseed = nullptr;  // cylinder layout (lazy)
    uint32_t* counts = nullptr;
    uint32_t* tested = nullptr;  // per-spin scanned grid entries (lazy)
    uint32_t* status = nullptr;
    float4* draws = nullptr;    // replay buffer (lazy, grows)
    size_t drawsCap = 0;
    float4* grad = nullptr;     // per-step gradient table (lazy, grows)
    size_t gradCap = 0;
    double* partials = nullptr; // signal scratch
    double* sig = nullptr;      // 15 doubles
    void* flush = nullptr;
    size_t flushCap = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    uint64_t bytes = 0;
    SpinsDev dev() const {
        SpinsDev S;
        S.x = x; S.y = y; S.z = z; S.mag = mag; S.phase = phase; S.meta = meta; S.seed = nullptr;
        S.N = N;
        return S;
    }
    SpinsSorted sorted() const {
        SpinsSorted S;
        S.x = x; S.y = y; S.z = z; S.mag = mag; S.phase = phase; S.meta = meta; S.id = id; S.N = N;
        return S;
    }
    SpinsSorted sorted2() const {
        SpinsSorted S;
        S.x = x2; S.y = y2; S.z = z2; S.mag = mag2; S.phase = phase2; S.meta = meta2; S.id = id2; S.N = N;
        return S;
    }
    void swap_buffers() {
        std::swap(x, x2); std::swap(y, y2); std::swap(z, z2); std::swap(mag, mag2);
        std::swap(phase, phase2); std::swap(meta, meta2); std::swap(id, id2);
    }
};

// ---------------------------------------------------------------------------
// mesh construction
// ---------------------------------------------------------------------------
static void mesh_release(dsim_mesh* m) {
    if (!m) return;
    cudaFree(m->V); cudaFree(m->trgls); cudaFree(m->membrane); cudaFree(m->fiber);
    cudaFree(m->plane); cudaFree(m->bary); cudaFree(m->cell_start); cudaFree(m->cell_tri); cudaFree(m->tri64);
    cudaFree(m->tri_cells);
    cudaFree(m->acc_start); cudaFree(m->acc_rec); cudaFree(m->acc_tri); cudaFree(m->acc_recw); cudaFree(m->acc_recf);
    delete m;
}

// Upload normalised vertices and triangles, compute records, build the grid.
static int mesh_build(dsim_mesh* m, const std::vector<float>& Vn, const std::vector<uint32_t>& trgls,
                      const std::vector<uint32_t>& membrane, const std::vector<uint32_t>& fiber) {
    int rc;
    m->nV = (uint32_t)(Vn.size() / 3);
    m->nT = (uint32_t)(trgls.size() / 3);
    for (uint32_t v = 0; v < m->nV; v++)
        for (int k = 0; k < 3; k++) m->maxabs[k] = fmaxf(fabsf(Vn[3 * v + k]), m->maxabs[k]);
    for (uint32_t t = 0; t < m->nT; t++)
        for (int k = 0; k < 3; k++)
            if (trgls[3 * t + k] >= m->nV) {
                set_last_error(kErrFormat, "triangle %u references vertex %u of %u", t, trgls[3 * t + k], m->nV);
                return kErrFormat;
            }
    if ((rc = dev_alloc(&m->V, Vn.size(), &m->bytes))) return rc;
    if ((rc = dev_alloc(&m->trgls, trgls.size(), &m->bytes))) return rc;
    if ((rc = dev_alloc(&m->membrane, m->nT, &m->bytes))) return rc;
    if ((rc = dev_alloc(&m->fiber, m->nT, &m->bytes))) return rc;
    if ((rc = dev_alloc(&m->plane, m->nT, &m->bytes))) return rc;
    if ((rc = dev_alloc(&m->bary, m->nT, &m->bytes))) return rc;
    cudaStream_t st = 0;
    DSIM_CUDA_TRY(cudaMemcpyAsync(m->V, Vn.data(), Vn.size() * 4, cudaMemcpyHostToDevice, st));
    DSIM_CUDA_TRY(cudaMemcpyAsync(m->trgls, trgls.data(), trgls.size() * 4, cudaMemcpyHostToDevice, st));
    if (m->nT) {
        DSIM_CUDA_TRY(cudaMemcpyAsync(m->membrane, membrane.data(), m->nT * 4, cudaMemcpyHostToDevice, st));
        DSIM_CUDA_TRY(cudaMemcpyAsync(m->fiber, fiber.data(), m->nT * 4, cudaMemcpyHostToDevice, st));
    }
    if ((rc = launch_records_from_mesh(m->nT, m->V, m->trgls, m->membrane, m->fiber, m->plane, m->bary, st)))
        return rc;
    // grid: count -> scan -> fill -> sort (populateCubes membership)
    uint32_t ncells = m->n * m->n * m->n;
    uint32_t* counter = nullptr;
    uint32_t* scratch = nullptr;
    if ((rc = dev_alloc(&counter, ncells))) return rc;
    if ((rc = dev_alloc(&scratch, scan_scratch_words(ncells)))) { cudaFree(counter); return rc; }
    if ((rc = dev_alloc(&m->cell_start, (size_t)ncells + 1, &m->bytes))) { cudaFree(counter); cudaFree(scratch); return rc; }
    rc = kOk;
    do {
        if (cudaMemsetAsync(counter, 0, ncells * 4, st) != cudaSuccess) { rc = kErrCuda; break; }
        if ((rc = launch_tri_cells(false, m->nT, m->V, m->trgls, m->n, m->L, counter, nullptr, nullptr, st))) break;
        if ((rc = launch_scan_exclusive(counter, m->cell_start, ncells, scratch, st))) break;
        uint32_t total = 0;
        if (cudaMemcpyAsync(&total, m->cell_start + ncells, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) { rc = kErrCuda; break; }
        m->entries = total;
        if ((rc = dev_alloc(&m->cell_tri, total, &m->bytes))) break;
        if (cudaMemsetAsync(counter, 0, ncells * 4, st) != cudaSuccess) { rc = kErrCuda; break; }
        if ((rc = launch_tri_cells(true, m->nT, m->V, m->trgls, m->n, m->L, counter, m->cell_start, m->cell_tri, st))) break;
        if ((rc = launch_sort_cells(ncells, m->cell_start, m->cell_tri, st))) break;
        if ((rc = dev_alloc(&m->tri_cells, m->nT, &m->bytes))) break;
        if (m->nT > ncells) {  // the scan scratch is sized for ncells; use a count of its own
            uint32_t* tcount = nullptr;
            if ((rc = dev_alloc(&tcount, m->nT))) break;
            rc = launch_tri_cell_lists(ncells, m->nT, m->cell_start, m->cell_tri, tcount, m->tri_cells, st);
            if (!rc && cudaStreamSynchronize(st) != cudaSuccess) rc = kErrCuda;
            cudaFree(tcount);
            if (rc) break;
        } else if ((rc = launch_tri_cell_lists(ncells, m->nT, m->cell_start, m->cell_tri, counter, m->tri_cells, st))) {
            break;
        }
        std::vector<uint32_t> cs(ncells + 1);
        if (cudaMemcpyAsync(cs.data(), m->cell_start, cs.size() * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) { rc = kErrCuda; break; }
        uint64_t mx = 0, ne = 0;
        for (uint32_t c = 0; c < ncells; c++) {
            uint32_t k = cs[c + 1] - cs[c];
            if (k > mx) mx = k;
            if (k) ne++;
        }
        m->maxPerCell = mx;
        m->nonempty = ne;
    } while (0);
    if (rc == kErrCuda) set_last_error(kErrCuda, "grid build: %s", cudaGetErrorString(cudaGetLastError()));
    cudaFree(counter);
    cudaFree(scratch);
    if (rc) return rc;
    // default fine grid: 2.25 fine cells per reference cell edge (50 -> 112)
    const uint32_t nf = 9 * m->n / 4;
    return accel_build(m, nf < 1 ? 1 : (nf <= 1024 ? nf : 1024));
}

extern "C" {

const char* dsim_last_error(void) { return last_error_message(); }
int dsim_version(void) { return 1; }

int dsim_device_info(char* name, int len, int* smCount, size_t* totalMem) {
    int dev = 0;
    DSIM_CUDA_TRY(cudaGetDevice(&dev));
    cudaDeviceProp p;
    DSIM_CUDA_TRY(cudaGetDeviceProperties(&p, dev));
    if (name && len > 0) { strncpy(name, p.name, len - 1); name[len - 1] = 0; }
    if (smCount) *smCount = p.multiProcessorCount;
    if (totalMem) *totalMem = p.totalGlobalMem;
    return kOk;
}

int dsim_mesh_load(const char* path, float spaceScale, uint32_t numCubes, dsim_mesh** out) {
    if (!path || !out || !(spaceScale > 0) || numCubes == 0 || numCubes > 1024) {
        set_last_error(kErrInvalid, "dsim_mesh_load: bad argument");
        return kErrInvalid;
    }
    *out = nullptr;
    MeshHost h;
    int rc = parse_mesh_file(path, spaceScale, h);
    if (rc) return rc;
    dsim_mesh* m = new dsim_mesh();
    m->n = numCubes;
    m->L = 2.0f / (float)numCubes;
    m->nFibers = h.nFibers;
    rc = mesh_build(m, h.vertices, h.trgls, h.membrane, h.fiber);
    if (rc) { mesh_release(m); return rc; }
    *out = m;
    return kOk;
}

int dsim_mesh_create(const float* vertices_um, uint32_t nVertices, const uint32_t* trgls,
                     const uint32_t* membrane, const uint32_t* fiber, uint32_t nTriangles,
                     float spaceScale, uint32_t numCubes, dsim_mesh** out) {
    if (!out || (!vertices_um && nVertices) || (!trgls && nTriangles) || !(spaceScale > 0) ||
        numCubes == 0 || numCubes > 1024) {
        set_last_error(kErrInvalid, "dsim_mesh_create: bad argument");
        return kErrInvalid;
    }
    *out = nullptr;
    std::vector<float> Vn((size_t)nVertices * 3);
    for (size_t k = 0; k < Vn.size(); k++) Vn[k] = vertices_um[k] / spaceScale;
    std::vector<uint32_t> T(trgls, trgls + (size_t)nTriangles * 3);
    std::vector<uint32_t> mem(nTriangles, 0u), fib(nTriangles, 0u);
    uint32_t nf = 0;
    for (uint32_t t = 0; t < nTriangles; t++) {
        mem[t] = membrane ? membrane[t] : 2u;
        fib[t] = fiber ? fiber[t] : 0u;
        if (mem[t] > 2u) { set_last_error(kErrInvalid, "membrane type %u > 2", mem[t]); return kErrInvalid; }
        if (fib[t] + 1 > nf) nf = fib[t] + 1;
    }
    dsim_mesh* m = new dsim_mesh();
    m->n = numCubes;
    m->L = 2.0f / (float)numCubes;
    m->nFibers = nf;
    int rc = mesh_build(m, Vn, T, mem, fib);
    if (rc) { mesh_release(m); return rc; }
    *out = m;
    return kOk;
}

int dsim_mesh_accel_info(const dsim_mesh* m, uint64_t info[3]) {
    if (!m || !info) return kErrInvalid;
    info[0] = m->nf; info[1] = m->accEntries; info[2] = m->accBytes;
    return kOk;
}

int dsim_mesh_info(const dsim_mesh* m, uint64_t info[8]) {
    if (!m || !info) return kErrInvalid;
    info[0] = m->nV; info[1] = m->nT; info[2] = m->nFibers; info[3] = m->n;
    info[4] = m->entries; info[5] = m->maxPerCell; info[6] = m->bytes; info[7] = m->nonempty;
    return kOk;
}

int dsim_mesh_grid(const dsim_mesh* m, uint32_t* cellStart, uint32_t* cellTri) {
    if (!m) return kErrInvalid;
    size_t nc = (size_t)m->n * m->n * m->n;
    if (cellStart) DSIM_CUDA_TRY(cudaMemcpy(cellStart, m->cell_start, (nc + 1) * 4, cudaMemcpyDeviceToHost));
    if (cellTri && m->entries) DSIM_CUDA_TRY(cudaMemcpy(cellTri, m->cell_tri, m->entries * 4, cudaMemcpyDeviceToHost));
    return kOk;
}

int dsim_mesh_arrays(const dsim_mesh* m, float* vertices, uint32_t* triInfo) {
    if (!m) return kErrInvalid;
    if (vertices && m->nV) DSIM_CUDA_TRY(cudaMemcpy(vertices, m->V, (size_t)m->nV * 12, cudaMemcpyDeviceToHost));
    if (triInfo && m->nT) {
        std::vector<uint32_t> T((size_t)m->nT * 3), mem(m->nT), fib(m->nT);
        DSIM_CUDA_TRY(cudaMemcpy(T.data(), m->trgls, T.size() * 4, cudaMemcpyDeviceToHost));
        DSIM_CUDA_TRY(cudaMemcpy(mem.data(), m->membrane, m->nT * 4, cudaMemcpyDeviceToHost));
        DSIM_CUDA_TRY(cudaMemcpy(fib.data(), m->fiber, m->nT * 4, cudaMemcpyDeviceToHost));
        for (uint32_t t = 0; t < m->nT; t++) {
            triInfo[3 * t] = fib[t]; triInfo[3 * t + 1] = mem[t]; triInfo[3 * t + 2] = T[3 * t];
        }
    }
    return kOk;
}

void dsim_mesh_free(dsim_mesh* m) { mesh_release(m); }

// ---------------------------------------------------------------------------
// cylinders
// ---------------------------------------------------------------------------
static void cyl_fine_release(dsim_cyl* c) {
    cudaFree(c->fineStart); cudaFree(c->fineRec); cudaFree(c->finePos);
    c->fineStart = nullptr; c->fineRec = nullptr; c->finePos = nullptr;
    c->bytes -= c->fineBytes;
    c->fineK = 0; c->fineEntries = 0; c->fineBytes = 0;
}

static int cyl_holds(const dsim_cyl* c) {
    std::lock_guard<std::mutex> lk(g_cylHoldMu);
    auto it = g_cylHolds.find(c);
    return it == g_cylHolds.end() ? 0 : it->second;
}

static void cyl_release(dsim_cyl* c) {
    if (!c) return;
    {
        std::lock_guard<std::mutex> lk(g_cylHoldMu);
        g_cylHolds.erase(c);
    }
    cudaFree(c->fibers); cudaFree(c->cc); cudaFree(c->cubes); cudaFree(c->cubeF);
    cyl_fine_release(c);
    delete c;
}

// Fine filter grid.  A spin outside every fiber tests the entries of its
// grid cell's list in order, and only an entry whose fiber disk holds the
// tested point (d^2 <= r^2, or d^2 < inR r^2 with inR <= 1) changes anything.
// Each grid cell is split k x k x k; a fine cell keeps, in list order and
// with repeats, the list positions whose disk can reach the cell: in double,
// d^2 from the axis to the cell's box widened by 1e-5 at most r^2 (1 + 1e-4)
// (the float distance of a point within the box is far inside that margin),
// with the boxes of the outermost fine cells reaching to infinity outward
// (a proposed position can leave the box before the clamp; the grid cell of
// such a point is the clamped one).  The spin's fine cell is taken inside
// its grid cell, so the fine list is a subsequence of the list it replaces.
static uint32_t cyl_fine_default(const CylHost& h) {
    return cyl_fine_size(h.numCubes, h.cubeLength, h.maxR);
}

static int cyl_fine_build(dsim_cyl* c, uint32_t k) {
    cyl_fine_release(c);
    const CylHost& h = c->host;
    if (k < 2 || h.numCubes == 0 || !c->cubeF) return kOk;
    std::vector<uint32_t> start, pos;
    std::vector<float> rec;
    int rc = dsim::cyl_fine_lists(h.fiberPos.data(), h.nF, h.numCubes, h.maxFPC, h.cubeLength, h.cubeCounter.data(),
                            h.cubes.data(), k, start, pos, rec);
    if (rc) return rc;
    const size_t nfine = start.size() - 1;
    if ((rc = dev_alloc(&c->fineStart, nfine + 1, &c->fineBytes)) || (rc = dev_alloc(&c->fineRec, pos.size(), &c->fineBytes)) ||
        (rc = dev_alloc(&c->finePos, pos.size(), &c->fineBytes))) {
        cyl_fine_release(c);
        return rc;
    }
    c->bytes += c->fineBytes;
    DSIM_CUDA_TRY(cudaMemcpy(c->fineStart, start.data(), start.size() * 4, cudaMemcpyHostToDevice));
    if (!pos.empty()) {
        DSIM_CUDA_TRY(cudaMemcpy(c->fineRec, rec.data(), rec.size() * 4, cudaMemcpyHostToDevice));
        DSIM_CUDA_TRY(cudaMemcpy(c->finePos, pos.data(), pos.size() * 4, cudaMemcpyHostToDevice));
    }
    c->fineK = k;
    c->fineEntries = pos.size();
    return kOk;
}

// the fibers on the device, the reference's grid built there (addEntities,
// cyl.cu) with each entry's fiber record inline, host mirrors of the grid for
// the fine lists and dsim_cyl_info, then the fine filter grid
static int cyl_upload(dsim_cyl* c) {
    int rc;
    CylHost& h = c->host;
    if ((rc = cyl_grid_geometry(h))) return rc;
    const size_t ncells = (size_t)h.numCubes * h.numCubes * h.numCubes;
    const size_t slots = std::max<size_t>(1, ncells * h.maxFPC);
    if ((rc = dev_alloc(&c->fibers, std::max<uint32_t>(1, h.nF), &c->bytes))) return rc;
    if ((rc = dev_alloc(&c->cc, ncells, &c->bytes))) return rc;
    if ((rc = dev_alloc(&c->cubes, slots, &c->bytes))) return rc;
    if ((rc = dev_alloc(&c->cubeF, slots, &c->bytes))) return rc;
    if (h.nF) DSIM_CUDA_TRY(cudaMemcpy(c->fibers, h.fiberPos.data(), (size_t)h.nF * 16, cudaMemcpyHostToDevice));
    uint32_t mx = 0;
    if ((rc = build_cyl_grid_gpu(c->fibers, h.nF, h.numCubes, h.maxFPC, h.cubeLength, h.maxR, c->cc, c->cubes,
                                 c->cubeF, &mx, 0)))
        return rc;
    h.cubeCounter.resize(ncells);
    h.cubes.resize(ncells * h.maxFPC);
    DSIM_CUDA_TRY(cudaMemcpy(h.cubeCounter.data(), c->cc, ncells * 4, cudaMemcpyDeviceToHost));
    if (!h.cubes.empty())
        DSIM_CUDA_TRY(cudaMemcpy(h.cubes.data(), c->cubes, h.cubes.size() * 4, cudaMemcpyDeviceToHost));
    if ((rc = cyl_fine_build(c, cyl_fine_default(h)))) return rc;
    return kOk;
}

int dsim_cyl_load(const char* path, float spaceScale, dsim_cyl** out) {
    if (!path || !out || !(spaceScale > 0)) { set_last_error(kErrInvalid, "dsim_cyl_load: bad argument"); return kErrInvalid; }
    *out = nullptr;
    dsim_cyl* c = new dsim_cyl();
    int rc = parse_cyl_file(path, spaceScale, c->host);
    if (!rc) rc = cyl_upload(c);
    if (rc) { cyl_release(c); return rc; }
    *out = c;
    return kOk;
}

int dsim_cyl_create(const float* fiberPos4, uint32_t nFibers, float maxRadius, dsim_cyl** out) {
    if (!out || (!fiberPos4 && nFibers) || !(maxRadius > 0)) { set_last_error(kErrInvalid, "dsim_cyl_create: bad argument"); return kErrInvalid; }
    *out = nullptr;
    dsim_cyl* c = new dsim_cyl();
    c->host.nF = nFibers;
    c->host.fiberPos.assign(fiberPos4, fiberPos4 + (size_t)nFibers * 4);
    c->host.maxR = maxRadius;
    int rc = cyl_upload(c);
    if (rc) { cyl_release(c); return rc; }
    *out = c;
    return kOk;
}

int dsim_cyl_info(const dsim_cyl* c, uint32_t geom[3], float* cubeLength, uint32_t* cubeCounter,
                  uint32_t* cubes, float* fiberPos4) {
    if (!c) return kErrInvalid;
    const CylHost& h = c->host;
    if (geom) { geom[0] = h.numCubes; geom[1] = h.maxFPC; geom[2] = h.nF; }
    if (cubeLength) *cubeLength = h.cubeLength;
    if (cubeCounter) memcpy(cubeCounter, h.cubeCounter.data(), h.cubeCounter.size() * 4);
    if (cubes && !h.cubes.empty()) memcpy(cubes, h.cubes.data(), h.cubes.size() * 4);
    if (fiberPos4 && h.nF) memcpy(fiberPos4, h.fiberPos.data(), (size_t)h.nF * 16);
    return kOk;
}

int dsim_cyl_set_fine(dsim_cyl* c, uint32_t k) {
    if (!c) return kErrInvalid;
    if (cyl_holds(c) > 0) {
        set_last_error(kErrInvalid, "dsim_cyl_set_fine: the substrate is in a batch (free the batch first)");
        return kErrInvalid;
    }
    return cyl_fine_build(c, k);
}

int dsim_cyl_fine_lists(const float* fiberPos4, uint32_t nFibers, uint32_t numCubes, uint32_t maxFibersPerCube,
                        float cubeLength, const uint32_t* cubeCounter, const uint32_t* cubes, uint32_t k,
                        uint32_t* start, uint32_t* positions, uint64_t capacity, uint64_t* entries) {
    if (!fiberPos4 || !cubeCounter || !cubes || !entries) { set_last_error(kErrInvalid, "dsim_cyl_fine_lists: null argument"); return kErrInvalid; }
    std::vector<uint32_t> st, pos;
    std::vector<float> rec;
    int rc = dsim::cyl_fine_lists(fiberPos4, nFibers, numCubes, maxFibersPerCube, cubeLength, cubeCounter, cubes, k, st,
                                  pos, rec);
    if (rc) return rc;
    *entries = pos.size();
    if (start) memcpy(start, st.data(), st.size() * 4);
    if (positions) {
        if (pos.size() > capacity) {
            set_last_error(kErrTooLarge, "dsim_cyl_fine_lists: %zu entries, capacity %llu", pos.size(), (unsigned long long)capacity);
            return kErrTooLarge;
        }
        if (!pos.empty()) memcpy(positions, pos.data(), pos.size() * 4);
    }
    return kOk;
}

int dsim_cyl_fine_info(const dsim_cyl* c, uint64_t info[3]) {
    if (!c || !info) return kErrInvalid;
    info[0] = c->fineK; info[1] = c->fineEntries; info[2] = c->fineBytes;
    return kOk;
}

void dsim_cyl_free(dsim_cyl* c) { cyl_release(c); }

// ---------------------------------------------------------------------------
// spins
// ---------------------------------------------------------------------------
static void spins_release(dsim_spins* s) {
    if (!s) return;
    if (s->st) cudaStreamSynchronize(s->st);
    cudaFree(s->x); cudaFree(s->y); cudaFree(s->z); cudaFree(s->mag); cudaFree(s->phase);
    cudaFree(s->meta); cudaFree(s->cpos); cudaFree(s->cseed); cudaFree(s->counts);
    cudaFree(s->status); cudaFree(s->tested); cudaFree(s->draws); cudaFree(s->grad); cudaFree(s->partials);
    cudaFree(s->sig); cudaFree(s->flush);
    cudaFree(s->id); cudaFree(s->x2); cudaFree(s->y2); cudaFree(s->z2); cudaFree(s->mag2);
    cudaFree(s->phase2); cudaFree(s->meta2); cudaFree(s->id2); cudaFree(s->keys); cudaFree(s->hist);
    cudaFree(s->hstart); cudaFree(s->hscratch);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->st) cudaStreamDestroy(s->st);
    delete s;
}

int dsim_spins_create(uint32_t N, dsim_spins** out) {
    if (!out) return kErrInvalid;
    *out = nullptr;
    dsim_spins* s = new dsim_spins();
    s->N = N;
    int rc = kOk;
    do {
        if (cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) != cudaSuccess) { rc = kErrCuda; break; }
        if (cudaEventCreate(&s->ev0) != cudaSuccess || cudaEventCreate(&s->ev1) != cudaSuccess) { rc = kErrCuda; break; }
        if ((rc = dev_alloc(&s->x, N, &s->bytes)) || (rc = dev_alloc(&s->y, N, &s->bytes)) ||
            (rc = dev_alloc(&s->z, N, &s->bytes)) || (rc = dev_alloc(&s->mag, N, &s->bytes)) ||
            (rc = dev_alloc(&s->phase, N, &s->bytes)) || (rc = dev_alloc(&s->meta, N, &s->bytes)) ||
            (rc = dev_alloc(&s->counts, (size_t)2 * N, &s->bytes)) || (rc = dev_alloc(&s->status, 1, &s->bytes)) ||
            (rc = dev_alloc(&s->partials, reduce_scratch_doubles(N), &s->bytes)) ||
            (rc = dev_alloc(&s->sig, 15, &s->bytes)) || (rc = dev_alloc(&s->id, N, &s->bytes)))
            break;
        if (cudaMemsetAsync(s->counts, 0, (size_t)8 * N, s->st) != cudaSuccess ||
            cudaMemsetAsync(s->status, 0, 4, s->st) != cudaSuccess) { rc = kErrCuda; break; }
        std::vector<uint32_t> iota(N);
        for (uint32_t i = 0; i < N; i++) iota[i] = i;
        if (cudaMemcpyAsync(s->id, iota.data(), (size_t)4 * N, cudaMemcpyHostToDevice, s->st) != cudaSuccess ||
            cudaStreamSynchronize(s->st) != cudaSuccess) { rc = kErrCuda; break; }
    } while (0);
    if (rc == kErrCuda) set_last_error(kErrCuda, "dsim_spins_create: %s", cudaGetErrorString(cudaGetLastError()));
    if (rc) { spins_release(s); return rc; }
    *out = s;
    return kOk;
}

uint32_t dsim_spins_count(const dsim_spins* s) { return s ? s->N : 0; }
uint64_t dsim_spins_bytes(const dsim_spins* s) { return s ? s->bytes : 0; }

static int spins_identity(dsim_spins* s) {
    std::vector<uint32_t> iota(s->N);
    for (uint32_t i = 0; i < s->N; i++) iota[i] = i;
    DSIM_CUDA_TRY(cudaMemcpyAsync(s->id, iota.data(), (size_t)4 * s->N, cudaMemcpyHostToDevice, s->st));
    DSIM_CUDA_TRY(cudaStreamSynchronize(s->st));
    s->permuted = false;
    return kOk;
}

// bring slot order back to spin order (slot i holds spin i)
static int spins_unpermute(dsim_spins* s) {
    if (!s->permuted) return kOk;
    int rc = launch_unpermute(s->sorted(), s->sorted2(), s->st);
    if (rc) return rc;
    s->launches += 1;
    s->swap_buffers();
    s->permuted = false;
    return kOk;
}

static int ensure_sort_buffers(dsim_spins* s, uint32_t nb) {
    int rc;
    if (!s->x2) {
        if ((rc = dev_alloc(&s->x2, s->N, &s->bytes)) || (rc = dev_alloc(&s->y2, s->N, &s->bytes)) ||
            (rc = dev_alloc(&s->z2, s->N, &s->bytes)) || (rc = dev_alloc(&s->mag2, s->N, &s->bytes)) ||
            (rc = dev_alloc(&s->phase2, s->N, &s->bytes)) || (rc = dev_alloc(&s->meta2, s->N, &s->bytes)) ||
            (rc = dev_alloc(&s->id2, s->N, &s->bytes)) || (rc = dev_alloc(&s->keys, s->N, &s->bytes)))
            return rc;
    }
    if (s->sortNb != nb) {
        cudaFree(s->hist); cudaFree(s->hstart); cudaFree(s->hscratch);
        s->hist = s->hstart = s->hscratch = nullptr;
        uint32_t nkeys = accel_keys(nb);
        if ((rc = dev_alloc(&s->hist, nkeys, &s->bytes)) || (rc = dev_alloc(&s->hstart, (size_t)nkeys + 1, &s->bytes)) ||
            (rc = dev_alloc(&s->hscratch, scan_scratch_words(nkeys), &s->bytes)))
            return rc;
        s->sortNb = nb;
    }
    return kOk;
}

int dsim_spins_set(dsim_spins* s, const float* pos3, const float* mag, const float* phase,
                   const uint8_t* comp, const uint16_t* fiber) {
    if (!s) return kErrInvalid;
    uint32_t N = s->N;
    int rc0 = spins_unpermute(s);
    if (rc0) return rc0;
    std::vector<float> a(N), b(N), c(N);
    if (pos3) {
        for (uint32_t i = 0; i < N; i++) { a[i] = pos3[3 * i]; b[i] = pos3[3 * i + 1]; c[i] = pos3[3 * i + 2]; }
        DSIM_CUDA_TRY(cudaMemcpyAsync(s->x, a.data(), N * 4, cudaMemcpyHostToDevice, s->st));
        DSIM_CUDA_TRY(cudaMemcpyAsync(s->y, b.data(), N * 4, cudaMemcpyHostToDevice, s->st));
        DSIM_CUDA_TRY(cudaMemcpyAsync(s->z, c.data(), N * 4, cudaMemcpyHostToDevice, s->st));
        DSIM_CUDA_TRY(cudaStreamSynchronize(s->st));
    }
    if (mag) DSIM_CUDA_TRY(cudaMemcpyAsync(s->mag, mag, N * 4, cudaMemcpyHostToDevice, s->st));
    if (phase) DSIM_CUDA_TRY(cudaMemcpyAsync(s->phase, phase, N * 4, cudaMemcpyHostToDevice, s->st));
    if (comp || fiber) {
        std::vector<uint32_t> m(N);
        for (uint32_t i = 0; i < N; i++)
            m[i] = (comp ? (uint32_t)comp[i] : 0u) | ((fiber ? (uint32_t)fiber[i] : 0xFFFFu) << 8);
        DSIM_CUDA_TRY(cudaMemcpyAsync(s->meta, m.data(), N * 4, cudaMemcpyHostToDevice, s->st));
        DSIM_CUDA_TRY(cudaStreamSynchronize(s->st));
    }
    DSIM_CUDA_TRY(cudaStreamSynchronize(s->st));
    return kOk;
}

int dsim_spins_get(dsim_spins* s, float* pos3, float* mag, float* phase, uint8_t* comp,
                   uint16_t* fiber) {
    if (!s) return kErrInvalid;
    uint32_t N = s->N;
    int rc0 = spins_unpermute(s);
    if (rc0) return rc0;
    if (pos3) {
        std::vector<float> a(N), b(N), c(N);
        DSIM_CUDA_TRY(cudaMemcpyAsync(a.data(), s->x, N * 4, cudaMemcpyDeviceToHost, s->st));
        DSIM_CUDA_TRY(cudaMemcpyAsync(b.data(), s->y, N * 4, cudaMemcpyDeviceToHost, s->st));
        DSIM_CUDA_TRY(cudaMemcpyAsync(c.data(), s->z, N * 4, cudaMemcpyDeviceToHost, s->st));
        DSIM_CUDA_TRY(cudaStreamSynchronize(s->st));
        for (uint32_t i = 0; i < N; i++) { pos3[3 * i] = a[i]; pos3[3 * i + 1] = b[i]; pos3[3 * i + 2] = c[i]; }
    }
    if (mag) DSIM_CUDA_TRY(cudaMemcpyAsync(mag, s->mag, N * 4, cudaMemcpyDeviceToHost, s->st));
    if (phase) DSIM_CUDA_TRY(cudaMemcpyAsync(phase, s->phase, N * 4, cudaMemcpyDeviceToHost, s->st));
    if (comp || fiber) {
        std::vector<uint32_t> m(N);
        DSIM_CUDA_TRY(cudaMemcpyAsync(m.data(), s->meta, N * 4, cudaMemcpyDeviceToHost, s->st));
        DSIM_CUDA_TRY(cudaStreamSynchronize(s->st));
        for (uint32_t i = 0; i < N; i++) {
            if (comp) comp[i] = (uint8_t)(m[i] & 0xFFu);
            if (fiber) fiber[i] = (uint16_t)(m[i] >> 8);
        }
    }
    DSIM_CUDA_TRY(cudaStreamSynchronize(s->st));
    return kOk;
}

static int ensure_cyl(dsim_spins* s) {
    int rc;
    if (!s->cpos && (rc = dev_alloc(&s->cpos, s->N, &s->bytes))) return rc;
    if (!s->cseed && (rc = dev_alloc(&s->cseed, (size_t)4 * s->N, &s->bytes))) return rc;
    return kOk;
}

int dsim_spins_set_cyl(dsim_spins* s, const float* pos3, const float* mag, const float* phase,
                       const uint32_t* imo, const uint32_t* nearest) {
    if (!s || !pos3) return kErrInvalid;
    int rc = ensure_cyl(s);
    if (rc) return rc;
    uint32_t N = s->N;
    std::vector<float4> p(N);
    std::vector<uint32_t> sd((size_t)4 * N, 0u);
    for (uint32_t i = 0; i < N; i++) {
        p[i] = make_float4(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2], phase ? phase[i] : 0.0f);
        sd[4 * i + 2] = (imo ? imo[i] : 2u) + 1u;
        sd[4 * i + 3] = nearest ? nearest[i] : 0xFFFFFFFFu;
    }
    DSIM_CUDA_TRY(cudaMemcpyAsync(s->cpos, p.data(), (size_t)N * 16, cudaMemcpyHostToDevice, s->st));
    DSIM_CUDA_TRY(cudaMemcpyAsync(s->cseed, sd.data(), (size_t)N * 16, cudaMemcpyHostToDevice, s->st));
    if (mag) DSIM_CUDA_TRY(cudaMemcpyAsync(s->mag, mag, N * 4, cudaMemcpyHostToDevice, s->st));
    else {
        std::vector<float> one(N, 1.0f);
        DSIM_CUDA_TRY(cudaMemcpyAsync(s->mag, one.data(), N * 4, cudaMemcpyHostToDevice, s->st));
        DSIM_CUDA_TRY(cudaStreamSynchronize(s->st));
    }
    DSIM_CUDA_TRY(cudaStreamSynchronize(s->st));
    return kOk;
}

int dsim_spins_get_cyl(dsim_spins* s, float* pos3, float* mag, float* phase, uint32_t* imo,
                       uint32_t* nearest) {
    if (!s || !s->cpos) return kErrInvalid;
    uint32_t N = s->N;
    std::vector<float4> p(N);
    std::vector<uint32_t> sd((size_t)4 * N);
    DSIM_CUDA_TRY(cudaMemcpyAsync(p.data(), s->cpos, (size_t)N * 16, cudaMemcpyDeviceToHost, s->st));
    DSIM_CUDA_TRY(cudaMemcpyAsync(sd.data(), s->cseed, (size_t)N * 16, cudaMemcpyDeviceToHost, s->st));
    if (mag) DSIM_CUDA_TRY(cudaMemcpyAsync(mag, s->mag, N * 4, cudaMemcpyDeviceToHost, s->st));
    DSIM_CUDA_TRY(cudaStreamSynchronize(s->st));
    for (uint32_t i = 0; i < N; i++) {
        if (pos3) { pos3[3 * i] = p[i].x; pos3[3 * i + 1] = p[i].y; pos3[3 * i + 2] = p[i].z; }
        if (phase) phase[i] = p[i].w;
        if (imo) imo[i] = sd[4 * i + 2] ? sd[4 * i + 2] - 1u : 2u;
        if (nearest) nearest[i] = sd[4 * i + 3];
    }
    return kOk;
}

int dsim_spins_counts(dsim_spins* s, uint32_t* counts2N, int reset) {
    if (!s) return kErrInvalid;
    if (counts2N) {
        DSIM_CUDA_TRY(cudaMemcpyAsync(counts2N, s->counts, (size_t)8 * s->N, cudaMemcpyDeviceToHost, s->st));
    }
    if (reset) DSIM_CUDA_TRY(cudaMemsetAsync(s->counts, 0, (size_t)8 * s->N, s->st));
    DSIM_CUDA_TRY(cudaStreamSynchronize(s->st));
    return kOk;
}

int dsim_spins_scanned(dsim_spins* s, uint32_t* scannedN, int reset) {
    if (!s) return kErrInvalid;
    if (!s->tested) {
        if (scannedN) memset(scannedN, 0, (size_t)4 * s->N);
        return kOk;
    }
    if (scannedN) DSIM_CUDA_TRY(cudaMemcpyAsync(scannedN, s->tested, (size_t)4 * s->N, cudaMemcpyDeviceToHost, s->st));
    if (reset) DSIM_CUDA_TRY(cudaMemsetAsync(s->tested, 0, (size_t)4 * s->N, s->st));
    DSIM_CUDA_TRY(cudaStreamSynchronize(s->st));
    return kOk;
}

int dsim_spins_status(dsim_spins* s, uint32_t* status, int reset) {
    if (!s) return kErrInvalid;
    uint32_t v = 0;
    DSIM_CUDA_TRY(cudaMemcpyAsync(&v, s->status, 4, cudaMemcpyDeviceToHost, s->st));
    if (reset) DSIM_CUDA_TRY(cudaMemsetAsync(s->status, 0, 4, s->st));
    DSIM_CUDA_TRY(cudaStreamSynchronize(s->st));
    if (status) *status = v;
    return kOk;
}

void dsim_spins_free(dsim_spins* s) { spins_release(s); }

// ---------------------------------------------------------------------------
// runs
// ---------------------------------------------------------------------------
static int upload_grad_draws(dsim_spins* s, const float* gradPerStep, const float* replayDraws,
                             uint32_t iterations, const float4** gradDev, const float4** drawsDev) {
    int rc;
    *gradDev = nullptr;
    *drawsDev = nullptr;
    if (gradPerStep) {
        if (s->gradCap < iterations) {
            cudaFree(s->grad); s->grad = nullptr; s->gradCap = 0;
            if ((rc = dev_alloc(&s->grad, iterations))) return rc;
            s->gradCap = iterations;
        }
        std::vector<float4> g(iterations);
        for (uint32_t k = 0; k < iterations; k++)
            g[k] = make_float4(gradPerStep[3 * k], gradPerStep[3 * k + 1], gradPerStep[3 * k + 2], 0.0f);
        DSIM_CUDA_TRY(cudaMemcpyAsync(s->grad, g.data(), (size_t)iterations * 16, cudaMemcpyHostToDevice, s->st));
        DSIM_CUDA_TRY(cudaStreamSynchronize(s->st));
        *gradDev = s->grad;
    }
    if (replayDraws) {
        size_t need = (size_t)iterations * s->N;
        if (s->drawsCap < need) {
            cudaFree(s->draws); s->draws = nullptr; s->drawsCap = 0;
            if ((rc = dev_alloc(&s->draws, need))) return rc;
            s->drawsCap = need;
        }
        DSIM_CUDA_TRY(cudaMemcpyAsync(s->draws, replayDraws, need * 16, cudaMemcpyHostToDevice, s->st));
        *drawsDev = s->draws;
    }
    return kOk;
}

int dsim_mesh_run(dsim_mesh* m, dsim_spins* s, const dsim_mesh_params* p, const float g[3],
                  const float* gradPerStep, uint32_t iterations, uint64_t seed, uint64_t step0,
                  const float* replayDraws, int countCollisions) {
    if (!m || !s || !p) { set_last_error(kErrInvalid, "dsim_mesh_run: null argument"); return kErrInvalid; }
    MeshStepArgs a;
    memset(&a, 0, sizeof(a));
    for (int k = 0; k < 4; k++) { a.sd[k] = p->stdDevs[k]; a.T2[k] = p->T2[k]; }
    a.perm = p->permeability;
    a.reflType = p->reflectionType;
    a.clampHi = 1.0f - p->spinRadius;
    a.clampLo = -1.0f + p->spinRadius;
    a.dt = p->deltaTime;
    a.pc = p->phaseConstant;
    if (g) { a.gx = g[0]; a.gy = g[1]; a.gz = g[2]; }
    a.iterations = iterations;
    a.key0 = (uint32_t)seed; a.key1 = (uint32_t)(seed >> 32);
    a.step0 = step0;
    a.stream = 0;
    a.maxSub = p->maxSubsegments ? p->maxSubsegments : 4096u;
    a.status = s->status;
    a.spinBase = s->spinBase;
    a.counts = (countCollisions & 1) ? s->counts : nullptr;
    if (countCollisions & 2) {
        if (!s->tested) {
            int rc0 = dev_alloc(&s->tested, s->N, &s->bytes);
            if (rc0) return rc0;
            DSIM_CUDA_TRY(cudaMemsetAsync(s->tested, 0, (size_t)4 * s->N, s->st));
        }
        a.tested = s->tested;
    }
    int rc = upload_grad_draws(s, gradPerStep, replayDraws, iterations, &a.grad, &a.draws);
    if (rc) return rc;
    int rng = replayDraws ? kRngReplay : kRngPhilox;
    if (m->nf == 0) {
        set_last_error(kErrInvalid, "dsim_mesh_run: the mesh has no fine grid (dsim_mesh_set_accel failed)");
        return kErrInvalid;
    }
    // reorder by fine cell every sortEvery steps
    uint32_t chunk = s->sortEvery ? s->sortEvery : iterations;
    if (s->sortEvery && (rc = ensure_sort_buffers(s, m->nf))) return rc;
    const float4* grad0 = a.grad;
    const float4* draws0 = a.draws;
    for (uint32_t done = 0; done < iterations; done += chunk) {
        uint32_t n = iterations - done < chunk ? iterations - done : chunk;
        if (s->sortEvery) {
            if ((rc = launch_sort_spins(s->sorted(), s->sorted2(), s->sortNb, s->keys, s->hist,
                                        s->hstart, s->hscratch, s->st)))
                return rc;
            s->launches += 5;  // keys, scan (3), scatter
            s->swap_buffers();
            s->permuted = true;
        }
        MeshStepArgs b = a;
        b.iterations = n;
        b.step0 = a.step0 + done;
        b.grad = grad0 ? grad0 + done : nullptr;
        b.draws = draws0 ? draws0 + (size_t)done * s->N : nullptr;
        rc = launch_mesh_step_flat(m->dev(), m->acc(), b, s->sorted(), rng, s->st,
                                   m->kernel == 5 ? 8 : (m->kernel == 7 ? 4 : 6), m->kernel == 8, m->kernel == 9);
        if (rc) return rc;
        s->launches += 1;
    }
    return kOk;
}

int dsim_mesh_set_kernel(dsim_mesh* m, uint32_t variant) {
    if (!m || variant < 5 || variant > 9) { set_last_error(kErrInvalid, "kernel variant must be 5..9"); return kErrInvalid; }
    m->kernel = variant;
    return kOk;
}

int dsim_mesh_set_accel(dsim_mesh* m, uint32_t cellsPerAxis) {
    if (!m) return kErrInvalid;
    if (cellsPerAxis == 0) {
        set_last_error(kErrInvalid, "dsim_mesh_set_accel: every step kernel needs a fine grid (cells per axis >= 1)");
        return kErrInvalid;
    }
    return accel_build(m, cellsPerAxis);
}

int dsim_mesh_set_records(dsim_mesh* m, uint32_t bytesPerRecord) {
    if (!m || (bytesPerRecord != 16 && bytesPerRecord != 32 && bytesPerRecord != 64)) {
        set_last_error(kErrInvalid, "record size must be 16, 32 or 64 bytes");
        return kErrInvalid;
    }
    m->accWide = bytesPerRecord == 64 ? 2u : (bytesPerRecord == 32 ? 1u : 0u);
    return accel_build(m, m->nf);
}

int dsim_spins_set_sort_interval(dsim_spins* s, uint32_t steps) {
    if (!s) return kErrInvalid;
    s->sortEvery = steps;
    return kOk;
}

int dsim_cyl_run(dsim_cyl* c, dsim_spins* s, const dsim_cyl_params* p, const float g[3],
                 const float* gradPerStep, uint32_t iterations, uint64_t seed, uint64_t step0,
                 const float* replayDraws, int countCollisions) {
    if (!c || !s || !p || !s->cpos) { set_last_error(kErrInvalid, "dsim_cyl_run: bad argument (cylinder state set?)"); return kErrInvalid; }
    CylStepArgs a;
    memset(&a, 0, sizeof(a));
    // SpinSystem::update dSim2/src/spinSystem.cpp:809-913 and cpuIntegrateSystem
    // dSim2/src/spinKernelCpu.cpp:2-20: ADC scaled by spaceScale^2, sd = sqrt(2 ADC dt)
    float ss2 = p->spaceScale * p->spaceScale;
    float intra = p->intraAdc / ss2, extra = p->extraAdc / ss2, myelin = p->myelinAdc / ss2;
    a.intraSd = sqrtf(2.0f * intra * p->deltaTime);
    a.extraSd = sqrtf(2.0f * extra * p->deltaTime);
    a.myelinSd = sqrtf(2.0f * myelin * p->deltaTime);
    a.T2fiber = p->T2fiber; a.T2myelin = p->T2myelin; a.T2outside = p->T2outside;
    a.perm = p->permeability;
    a.inRadPropSq = p->innerRadiusProportion * p->innerRadiusProportion;
    a.clampHi = 1.0f - p->spinRadius;
    a.clampLo = -1.0f + p->spinRadius;
    a.dt = p->deltaTime;
    a.pc = p->phaseConstant;
    if (g) { a.gx = g[0]; a.gy = g[1]; a.gz = g[2]; }
    a.iterations = iterations;
    a.key0 = (uint32_t)seed; a.key1 = (uint32_t)(seed >> 32);
    a.step0 = step0;
    a.status = s->status;
    a.spinBase = s->spinBase;
    a.counts = countCollisions ? s->counts : nullptr;
    int rc = upload_grad_draws(s, gradPerStep, replayDraws, iterations, &a.grad, &a.draws);
    if (rc) return rc;
    CylSpinsDev S;
    S.pos = s->cpos; S.seed4 = s->cseed; S.mag = s->mag; S.N = s->N;
    s->launches += 1;
    return launch_cyl_step(c->dev(), a, S, replayDraws ? kRngReplay : kRngPhilox, s->st);
}

int dsim_signal(dsim_spins* s, double region, double out[15]) {
    if (!s || !out) return kErrInvalid;
    SpinsDev S = s->dev();
    int layout = kLayoutSoA;
    if (s->cpos) {
        S.x = reinterpret_cast<float*>(s->cpos);
        S.meta = s->cseed;
        layout = 2;
    }
    int rc = launch_signal(S, layout, region, s->partials, s->sig, s->st);
    if (rc) return rc;
    DSIM_CUDA_TRY(cudaMemcpyAsync(out, s->sig, 15 * sizeof(double), cudaMemcpyDeviceToHost, s->st));
    DSIM_CUDA_TRY(cudaStreamSynchronize(s->st));
    return kOk;
}

int dsim_sync(dsim_spins* s) {
    if (!s) return kErrInvalid;
    DSIM_CUDA_TRY(cudaStreamSynchronize(s->st));
    DSIM_CUDA_TRY(cudaGetLastError());
    return kOk;
}

int dsim_timer_start(dsim_spins* s) {
    if (!s) return kErrInvalid;
    DSIM_CUDA_TRY(cudaEventRecord(s->ev0, s->st));
    return kOk;
}

int dsim_timer_stop(dsim_spins* s, float* ms) {
    if (!s) return kErrInvalid;
    DSIM_CUDA_TRY(cudaEventRecord(s->ev1, s->st));
    DSIM_CUDA_TRY(cudaEventSynchronize(s->ev1));
    float v = 0;
    DSIM_CUDA_TRY(cudaEventElapsedTime(&v, s->ev0, s->ev1));
    if (ms) *ms = v;
    return kOk;
}

int dsim_mesh_compartments(dsim_mesh* m, dsim_spins* s, uint64_t seed, float startBoxSize, uint32_t* moved) {
    if (!m || !s) { set_last_error(kErrInvalid, "dsim_mesh_compartments: null argument"); return kErrInvalid; }
    if (m->nf == 0) {
        set_last_error(kErrInvalid, "dsim_mesh_compartments: needs the fine grid");
        return kErrInvalid;
    }
    uint32_t* dmoved = nullptr;
    int rc = dev_alloc(&dmoved, 1);
    if (rc) return rc;
    cudaError_t e = cudaMemsetAsync(dmoved, 0, 4, s->st);
    if (e == cudaSuccess) {
        rc = launch_compartments(m->dev(), m->acc(), s->sorted(), m->maxabs, startBoxSize, seed, 20, 8, s->status,
                                 dmoved, s->st);
        uint32_t h = 0;
        if (!rc) e = cudaMemcpyAsync(&h, dmoved, 4, cudaMemcpyDeviceToHost, s->st);
        if (!rc && e == cudaSuccess) e = cudaStreamSynchronize(s->st);
        if (moved) *moved = h;
    }
    cudaFree(dmoved);
    if (rc) return rc;
    if (e != cudaSuccess) { set_last_cuda_error(e, "dsim_mesh_compartments", __FILE__, __LINE__); return kErrCuda; }
    return kOk;
}

int dsim_spins_set_spin_base(dsim_spins* s, uint32_t base) {
    if (!s) { set_last_error(kErrInvalid, "dsim_spins_set_spin_base: null argument"); return kErrInvalid; }
    if ((uint64_t)base + s->N > 0x100000000ull) { set_last_error(kErrTooLarge, "spin base + N exceeds 2^32"); return kErrTooLarge; }
    s->spinBase = base;
    return kOk;
}

int dsim_spins_launches(dsim_spins* s, uint64_t* n, int reset) {
    if (!s || !n) { set_last_error(kErrInvalid, "dsim_spins_launches: null argument"); return kErrInvalid; }
    *n = s->launches;
    if (reset) s->launches = 0;
    return kOk;
}

int dsim_flush_l2(dsim_spins* s, size_t bytes) {
    if (!s) return kErrInvalid;
    if (s->flushCap < bytes) {
        cudaFree(s->flush); s->flush = nullptr; s->flushCap = 0;
        if (cudaMalloc(&s->flush, bytes) != cudaSuccess) { cudaGetLastError(); set_last_error(kErrNoMem, "flush buffer"); return kErrNoMem; }
        s->flushCap = bytes;
    }
    DSIM_CUDA_TRY(cudaMemsetAsync(s->flush, s->flushCap & 0xFF, bytes, s->st));
    return kOk;
}

}  // extern "C"

namespace dsim {
int launch_rng_draws(uint64_t seed, uint32_t spin0, uint64_t step, uint32_t stream, uint32_t n,
                     uint32_t* raw, float* out, cudaStream_t st);
}

extern "C" int dsim_rng_draws(uint64_t seed, uint32_t spin0, uint64_t step, uint32_t stream,
                              uint32_t n, uint32_t* raw, float* draws4) {
    if (n == 0) return kOk;
    uint32_t* dRaw = nullptr;
    float* dOut = nullptr;
    int rc = dev_alloc(&dRaw, (size_t)4 * n);
    if (rc) return rc;
    if ((rc = dev_alloc(&dOut, (size_t)4 * n))) { cudaFree(dRaw); return rc; }
    rc = launch_rng_draws(seed, spin0, step, stream, n, dRaw, dOut, 0);
    if (!rc && raw && cudaMemcpy(raw, dRaw, (size_t)16 * n, cudaMemcpyDeviceToHost) != cudaSuccess) rc = kErrCuda;
    if (!rc && draws4 && cudaMemcpy(draws4, dOut, (size_t)16 * n, cudaMemcpyDeviceToHost) != cudaSuccess) rc = kErrCuda;
    if (rc == kErrCuda) set_last_error(kErrCuda, "dsim_rng_draws: %s", cudaGetErrorString(cudaGetLastError()));
    cudaFree(dRaw);
    cudaFree(dOut);
    return rc;
}
