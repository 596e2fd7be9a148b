// host_formats.cpp -- parsers for the reference's file formats and the
// reference's cylinder grid construction, on the host (setup code, not the
// hot path).  Semantics follow rfdougherty/dSim exactly so that the same
// files give the same substrate.
#include "host_formats.h"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "common.cuh"

namespace dsim {

static bool read_file(const char* path, std::string& out) {
    FILE* f = fopen(path, "rb");
    if (!f) return false;
    char buf[1 << 16];
    size_t n;
    out.clear();
    while ((n = fread(buf, 1, sizeof(buf), f)) > 0) out.append(buf, n);
    fclose(f);
    return true;
}

// Reader with the semantics of the fscanf calls in SpinSystem::initFibers:
// "%c" takes any next character; "%g" skips white space and converts a
// number, leaving the position at the first character it cannot use.
struct Scanner {
    const char* p;
    const char* end;
    bool eof() const { return p >= end; }
    bool getc(char& c) {
        if (p >= end) return false;
        c = *p++;
        return true;
    }
    bool getf(float& v) {
        while (p < end && isspace((unsigned char)*p)) p++;
        if (p >= end) return false;
        char* q = nullptr;
        // bounded copy: strtof needs a terminated string
        char tmp[64];
        size_t k = 0;
        while (p + k < end && k < sizeof(tmp) - 1 && !isspace((unsigned char)p[k])) { tmp[k] = p[k]; k++; }
        tmp[k] = 0;
        float x = strtof(tmp, &q);
        if (q == tmp) return false;
        p += (q - tmp);
        v = x;
        return true;
    }
};

// Two passes as in the reference: count blocks, then fill.  Block letters are
// recognised anywhere a single character is read (V, T, A<k>, M<k>, G<k>).
int parse_mesh_file(const char* path, float spaceScale, MeshHost& out) {
    std::string text;
    if (!read_file(path, text)) {
        set_last_error(kErrFile, "cannot open mesh file %s", path);
        return kErrFile;
    }
    out = MeshHost();
    uint32_t nV = 0, nT = 0;
    for (int pass = 0; pass < 2; pass++) {
        Scanner s{text.data(), text.data() + text.size()};
        uint32_t iv = 0, it = 0;
        char c;
        while (s.getc(c)) {
            if (c == 'V') {
                float x, y, z;
                for (;;) {
                    const char* save = s.p;
                    if (!s.getf(x)) break;
                    if (!s.getf(y) || !s.getf(z)) { (void)save; break; }
                    if (pass == 0) nV++;
                    else {
                        out.vertices[3 * iv + 0] = x / spaceScale;
                        out.vertices[3 * iv + 1] = y / spaceScale;
                        out.vertices[3 * iv + 2] = z / spaceScale;
                        out.maxabs[0] = fmaxf(fabsf(x) / spaceScale, out.maxabs[0]);
                        out.maxabs[1] = fmaxf(fabsf(y) / spaceScale, out.maxabs[1]);
                        out.maxabs[2] = fmaxf(fabsf(z) / spaceScale, out.maxabs[2]);
                        iv++;
                    }
                }
            } else if (c == 'T') {
                float a, b, d;
                for (;;) {
                    if (!s.getf(a)) break;
                    if (!s.getf(b) || !s.getf(d)) break;
                    if (pass == 0) nT++;
                    else {
                        out.trgls[3 * it + 0] = (uint32_t)a;
                        out.trgls[3 * it + 1] = (uint32_t)b;
                        out.trgls[3 * it + 2] = (uint32_t)d;
                        it++;
                    }
                }
            } else if (c == 'A' || c == 'M' || c == 'G') {
                uint32_t mem = (c == 'A') ? 0u : (c == 'M' ? 1u : 2u);
                if (pass == 0) {
                    if (mem == 0) out.nAxon++;
                    else if (mem == 1) out.nMyelin++;
                    else out.nGlia++;
                }
                float nr = 0.0f, tri;
                bool haveNr = s.getf(nr);
                uint32_t k = 0;
                while (s.getf(tri)) {
                    if (pass == 1) {
                        uint32_t t = (uint32_t)tri;
                        if (t >= nT) {
                            set_last_error(kErrFormat, "%s: membrane lists triangle %u of %u", path, t, nT);
                            return kErrFormat;
                        }
                        out.fiber[t] = haveNr ? (uint32_t)nr : 0u;
                        out.membrane[t] = mem;
                    }
                    k++;
                }
                if (pass == 0 && k > out.maxTrianglesOnSurface) out.maxTrianglesOnSurface = k;
            }
        }
        if (pass == 0) {
            if (out.nAxon != out.nMyelin) {
                // spinSystem.cpp:593-596: the reference exits here
                set_last_error(kErrFormat, "%s: %u axon and %u myelin membranes (must be equal)", path,
                               out.nAxon, out.nMyelin);
                return kErrFormat;
            }
            out.nFibers = out.nAxon + out.nGlia;
            out.vertices.assign((size_t)nV * 3, 0.0f);
            out.trgls.assign((size_t)nT * 3, 0u);
            out.membrane.assign(nT, 0u);
            out.fiber.assign(nT, 0u);
        }
    }
    return kOk;
}

// initFibers(FILE*), dSim2/src/spinSystem.cpp:323-385
int parse_cyl_file(const char* path, float spaceScale, CylHost& h) {
    FILE* fp = fopen(path, "r");
    if (!fp) {
        set_last_error(kErrFile, "cannot open cylinder file %s", path);
        return kErrFile;
    }
    h = CylHost();
    char str[256];
    float x, y, z, r;
    while (fgets(str, 255, fp) != NULL) {
        if (sscanf(str, "%f %f %f %f", &x, &y, &z, &r) == 4 &&
            (fabsf(x) + r < spaceScale || x == INFINITY) && (fabsf(y) + r < spaceScale || y == INFINITY) &&
            (fabsf(z) + r < spaceScale || z == INFINITY) && r > 0) {
            r = r / spaceScale;
            if (r > h.maxR) h.maxR = r;
            x = x / spaceScale; if (x > 2.0 || x == INFINITY) x = 2.0f;
            y = y / spaceScale; if (y > 2.0 || y == INFINITY) y = 2.0f;
            z = z / spaceScale; if (z > 2.0 || z == INFINITY) z = 2.0f;
            h.fiberPos.push_back(x);
            h.fiberPos.push_back(y);
            h.fiberPos.push_back(z);
            h.fiberPos.push_back(r * r);
            h.nF++;
        }
    }
    fclose(fp);
    return kOk;
}

// build() dSim2/src/spinSystem.cpp:135-228: the grid's size (cells per axis,
// list capacity, cell length); addEntities fills it on the GPU (cyl.cu)
int cyl_grid_geometry(CylHost& h) {
    if (!(h.maxR > 0.0f)) {
        set_last_error(kErrInvalid, "cylinder substrate has no fiber with positive radius");
        return kErrInvalid;
    }
    uint32_t t = (uint32_t)(2.0f / (float)(h.maxR * 4)) - 1;
    if (t < 2) t = 2;
    if (t > 100) t = 100;  // MAX_GRID_SIZE, dSim2/src/options.h:7
    h.numCubes = t;
    h.maxFPC = (uint32_t)ceil((double)(h.nF / (t * t) * 10));
    h.cubeLength = 2.0f / t;
    return kOk;
}

int parse_grads_file(const char* path, std::vector<GradRow>& rows) {
    FILE* f = fopen(path, "r");
    if (!f) {
        set_last_error(kErrFile, "cannot open gradient file %s", path);
        return kErrFile;
    }
    rows.clear();
    GradRow g;
    // readInputs, dSim3/src/diffusion.cpp:183-199: rows of six numbers
    while (!feof(f)) {
        int n = fscanf(f, "%g %g %g %g %g %g", &g.lDelta, &g.bDelta, &g.readOut, &g.gx, &g.gy, &g.gz);
        if (n == 6) rows.push_back(g);
        else if (n == EOF) break;
        else { int c = fgetc(f); if (c == EOF) break; }
    }
    fclose(f);
    return kOk;
}

}  // namespace dsim
