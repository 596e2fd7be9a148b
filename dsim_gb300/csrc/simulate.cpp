// simulate.cpp -- the reference's simulate call around the GPU path
// (include/dsim_sim.h): config and gradient files, PGSE sequencer, signal per
// gradient, diffusion-tensor fit, MATLAB results file.
//
// Reference: dSim3/src/diffusion.cpp (config 148-202, update() 522-737,
// computeTensor 286-511, writer 666-728); dSim2/src/diffusion.cpp (config
// 1095-1144, update() 183-287, writer header 1756-1770).
#include <cctype>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <map>
#include <string>
#include <vector>

#pragma GCC visibility push(default)
#include "../../include/dsim_batch.h"
#include "../../include/dsim_sim.h"
#pragma GCC visibility pop
#include "common.cuh"

using namespace dsim;

namespace {

// ---- libconfig subset -------------------------------------------------------
struct CfgParser {
    const std::string& s;
    size_t i = 0;
    std::map<std::string, std::string> kv;
    bool ok = true;
    explicit CfgParser(const std::string& text) : s(text) {}

    void skip() {
        for (;;) {
            while (i < s.size() && isspace((unsigned char)s[i])) i++;
            if (i + 1 < s.size() && s[i] == '/' && s[i + 1] == '/') {
                while (i < s.size() && s[i] != '\n') i++;
            } else if (i < s.size() && s[i] == '#') {
                while (i < s.size() && s[i] != '\n') i++;
            } else if (i + 1 < s.size() && s[i] == '/' && s[i + 1] == '*') {
                size_t e = s.find("*/", i + 2);
                i = (e == std::string::npos) ? s.size() : e + 2;
            } else {
                return;
            }
        }
    }
    std::string name() {
        skip();
        size_t b = i;
        while (i < s.size() && (isalnum((unsigned char)s[i]) || s[i] == '_' || s[i] == '-' || s[i] == '*')) i++;
        return s.substr(b, i - b);
    }
    // a scalar as text (strings without quotes; adjacent strings concatenate)
    bool scalar(std::string& out) {
        skip();
        if (i < s.size() && s[i] == '"') {
            out.clear();
            while (i < s.size() && s[i] == '"') {
                i++;
                while (i < s.size() && s[i] != '"') {
                    if (s[i] == '\\' && i + 1 < s.size()) i++;
                    out += s[i++];
                }
                if (i >= s.size()) return false;
                i++;
                skip();
            }
            return true;
        }
        size_t b = i;
        while (i < s.size() && !isspace((unsigned char)s[i]) && s[i] != ';' && s[i] != ',' && s[i] != ')' &&
               s[i] != ']' && s[i] != '}')
            i++;
        out = s.substr(b, i - b);
        return !out.empty();
    }
    bool value(const std::string& path) {
        skip();
        if (i >= s.size()) return false;
        if (s[i] == '{') {
            i++;
            if (!settings(path + ".")) return false;
            skip();
            if (i >= s.size() || s[i] != '}') return false;
            i++;
            return true;
        }
        if (s[i] == '(' || s[i] == '[') {
            const char close = s[i] == '(' ? ')' : ']';
            i++;
            int k = 0;
            for (;;) {
                skip();
                if (i < s.size() && s[i] == close) { i++; return true; }
                if (!value(path + "[" + std::to_string(k++) + "]")) return false;
                skip();
                if (i < s.size() && s[i] == ',') i++;
            }
        }
        std::string v;
        if (!scalar(v)) return false;
        kv[path] = v;
        return true;
    }
    bool settings(const std::string& prefix) {
        for (;;) {
            skip();
            if (i >= s.size() || s[i] == '}') return true;
            std::string n = name();
            if (n.empty()) return false;
            skip();
            if (i >= s.size() || (s[i] != '=' && s[i] != ':')) return false;
            i++;
            if (!value(prefix + n)) return false;
            skip();
            if (i < s.size() && (s[i] == ';' || s[i] == ',')) i++;
        }
    }
};

bool read_file(const char* path, std::string& out) {
    FILE* f = fopen(path, "rb");
    if (!f) return false;
    char buf[65536];
    size_t n;
    out.clear();
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) out.append(buf, n);
    fclose(f);
    return true;
}

void set_str(char* dst, const std::string& v) {
    strncpy(dst, v.c_str(), 511);
    dst[511] = 0;
}

// ---- gradient rows ------------------------------------------------------------
int parse_rows(const std::string& text, float* rows, uint32_t cap, uint32_t* n) {
    const char* p = text.c_str();
    std::vector<float> vals;
    for (;;) {
        while (*p && isspace((unsigned char)*p)) p++;
        if (!*p) break;
        char* e = nullptr;
        float v = strtof(p, &e);
        if (e == p) {
            set_last_error(kErrFormat, "gradient file: '%.20s' is not a number", p);
            return kErrFormat;
        }
        vals.push_back(v);
        p = e;
    }
    const uint32_t nr = (uint32_t)(vals.size() / 6);
    if (rows && nr > cap) { set_last_error(kErrTooLarge, "gradient file: %u rows > capacity %u", nr, cap); return kErrTooLarge; }
    if (rows) memcpy(rows, vals.data(), (size_t)nr * 6 * sizeof(float));
    *n = nr;
    return kOk;
}

// per-update counts of one run, as the reference rounds them
struct Sched {
    int lD, bD, ro, nUpdates;
};
Sched schedule(const float row[6], float timeStep, uint32_t spu) {
    const float per = timeStep * (float)spu;
    Sched s;
    s.lD = (int)(row[0] / per + 0.5);
    s.bD = (int)(row[1] / per + 0.5);
    s.ro = (int)(row[2] / per + 0.5);
    s.nUpdates = s.bD + s.lD + s.ro;
    return s;
}
// gradient factor (+1, 0, -1) for every update of one run
std::vector<float> update_signs(const Sched& s) {
    std::vector<float> w((size_t)std::max(s.nUpdates, 0), 0.0f);
    float g = 0.0f;
    for (int k = 0; k < s.nUpdates; k++) {
        if (k == 0) g = 1.0f;
        else if (k == s.lD && k < s.bD) g = 0.0f;
        else if (k == s.bD) g = -1.0f;
        else if (k == s.bD + s.lD) g = 0.0f;
        w[(size_t)k] = g;
    }
    return w;
}

// ---- tensor fit ---------------------------------------------------------------
void jacobi3(double a[3][3], double v[3][3], double d[3]) {
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) v[r][c] = (r == c) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 64; sweep++) {
        const double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
        if (off < 1e-300) break;
        for (int p = 0; p < 2; p++)
            for (int q = p + 1; q < 3; q++) {
                if (a[p][q] == 0.0) continue;
                const double th = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
                const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < 3; k++) {
                    const double akp = a[k][p], akq = a[k][q];
                    a[k][p] = c * akp - sn * akq;
                    a[k][q] = sn * akp + c * akq;
                }
                for (int k = 0; k < 3; k++) {
                    const double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = c * apk - sn * aqk;
                    a[q][k] = sn * apk + c * aqk;
                }
                for (int k = 0; k < 3; k++) {
                    const double vkp = v[k][p], vkq = v[k][q];
                    v[k][p] = c * vkp - sn * vkq;
                    v[k][q] = sn * vkp + c * vkq;
                }
            }
    }
    for (int k = 0; k < 3; k++) d[k] = a[k][k];
}

// Minimum-norm least squares through the eigen-decomposition of the 6 x 6
// normal matrix (cyclic Jacobi): directions whose singular value is below
// 1e-6 of the largest are dropped, as the reference's SVD pseudo-inverse
// (singular values rounded to 1e-6) drops them for rank-deficient tables.
bool solve6(double A[6][6], double b[6]) {
    const int n = 6;
    double V[6][6];
    for (int r = 0; r < n; r++)
        for (int c = 0; c < n; c++) V[r][c] = (r == c) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0, diag = 0.0;
        for (int p = 0; p < n; p++) {
            diag += A[p][p] * A[p][p];
            for (int q = p + 1; q < n; q++) off += A[p][q] * A[p][q];
        }
        if (off <= 1e-30 * diag) break;
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++) {
                if (A[p][q] == 0.0) continue;
                const double th = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
                const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < n; k++) {
                    const double akp = A[k][p], akq = A[k][q];
                    A[k][p] = c * akp - sn * akq;
                    A[k][q] = sn * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {
                    const double apk = A[p][k], aqk = A[q][k];
                    A[p][k] = c * apk - sn * aqk;
                    A[q][k] = sn * apk + c * aqk;
                }
                for (int k = 0; k < n; k++) {
                    const double vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = c * vkp - sn * vkq;
                    V[k][q] = sn * vkp + c * vkq;
                }
            }
    }
    double lmax = 0.0;
    for (int k = 0; k < n; k++) lmax = fmax(lmax, A[k][k]);
    if (!(lmax > 0.0)) return false;
    double x[6] = {0, 0, 0, 0, 0, 0};
    for (int k = 0; k < n; k++) {
        const double lam = A[k][k];
        if (lam <= 1e-12 * lmax) continue;  // singular value below 1e-6 of the largest
        double proj = 0.0;
        for (int r = 0; r < n; r++) proj += V[r][k] * b[r];
        for (int r = 0; r < n; r++) x[r] += V[r][k] * proj / lam;
    }
    for (int r = 0; r < n; r++) b[r] = x[r];
    return true;
}

// ---- cylinders: region and nearest fiber of a spin (dSim2 findNearestFiber,
// dSim2/src/spinSystem.cpp:1223-1311: the 3x3x3 cells around the spin) --------
uint32_t cyl_hash_host(float px, float py, float pz, float L, uint32_t n) {
    const float inv = 1.0f / L;
    float cx = floorf((px + 1.0f) * inv), cy = floorf((py + 1.0f) * inv), cz = floorf((pz + 1.0f) * inv);
    const float hi = (float)(n - 1);
    cx = fmaxf(fminf(cx, hi), 0.0f); cy = fmaxf(fminf(cy, hi), 0.0f); cz = fmaxf(fminf(cz, hi), 0.0f);
    return (uint32_t)((int)((float)(n * n) * cz) + (int)((float)n * cy) + (int)cx);
}
float cyl_dist_host(float px, float py, float pz, const float* f) {
    if (f[0] == 2.0f) return (pz - f[2]) * (pz - f[2]) + (py - f[1]) * (py - f[1]);
    if (f[2] == 2.0f) return (px - f[0]) * (px - f[0]) + (py - f[1]) * (py - f[1]);
    return (px - f[0]) * (px - f[0]) + (pz - f[2]) * (pz - f[2]);
}
void cyl_regions_host(const std::vector<float>& pos, const std::vector<float>& fp, const std::vector<uint32_t>& cc,
                      const std::vector<uint32_t>& cubes, uint32_t n, uint32_t maxFPC, float L, float inner,
                      std::vector<uint32_t>& imo, std::vector<uint32_t>& nearest) {
    const size_t N = pos.size() / 3;
    const float inSq = inner * inner;
    imo.assign(N, 2u);
    nearest.assign(N, 0xFFFFFFFFu);
    for (size_t s = 0; s < N; s++) {
        const float px = pos[3 * s], py = pos[3 * s + 1], pz = pos[3 * s + 2];
        float minD = 9.9e9f;
        for (int dy = -1; dy <= 1; dy++) {
            const float ty = py + dy * L;
            if (fabsf(ty) > 1.0f) continue;
            for (int dx = -1; dx <= 1; dx++) {
                const float tx = px + dx * L;
                if (fabsf(tx) > 1.0f) continue;
                for (int dz = -1; dz <= 1; dz++) {
                    const float tz = pz + dz * L;
                    if (fabsf(tz) > 1.0f) continue;
                    const uint32_t cube = cyl_hash_host(tx, ty, tz, L, n);
                    for (uint32_t j = 0; j < cc[cube]; j++) {
                        const uint32_t fi = cubes[(size_t)cube * maxFPC + j];
                        const float* f = &fp[4 * (size_t)fi];
                        const float d = cyl_dist_host(px, py, pz, f);
                        if (d < f[3]) imo[s] = (d < inSq * f[3]) ? 0u : 1u;
                        if (d < minD) { nearest[s] = fi; minD = d; }
                    }
                }
            }
        }
    }
}

// uniform positions in [-box, box]^3 from Philox (spin i of run `run`)
std::vector<float> reset_positions(uint32_t N, uint64_t seed, uint32_t run, float box) {
    std::vector<float> pos(3 * (size_t)N);
    for (uint32_t i = 0; i < N; i++) {
        const u32x4 r = philox4x32_10({i, run, 0u, 0x5E7u}, (uint32_t)seed, (uint32_t)(seed >> 32));
        pos[3 * (size_t)i] = box * 2.0f * ((float)(r.x >> 8) * 0x1p-24f - 0.5f);
        pos[3 * (size_t)i + 1] = box * 2.0f * ((float)(r.y >> 8) * 0x1p-24f - 0.5f);
        pos[3 * (size_t)i + 2] = box * 2.0f * ((float)(r.z >> 8) * 0x1p-24f - 0.5f);
    }
    return pos;
}

double sig_of(const double* sums, int c) {
    const double n = sums[3 * c + 2];
    return n > 0 ? std::sqrt(sums[3 * c] * sums[3 * c] + sums[3 * c + 1] * sums[3 * c + 1]) / n : 0.0;
}

bool file_exists(const std::string& p) {
    FILE* f = fopen(p.c_str(), "rb");
    if (!f) return false;
    fclose(f);
    return true;
}
std::string resolve(const std::string& cfgPath, const std::string& name) {
    if (name.empty() || name[0] == '/' || file_exists(name)) return name;
    const size_t slash = cfgPath.find_last_of('/');
    if (slash == std::string::npos) return name;
    const std::string alt = cfgPath.substr(0, slash + 1) + name;
    return file_exists(alt) ? alt : name;
}

}  // namespace

extern "C" {

int dsim_config_load(const char* path, dsim_config* out) {
    if (!path || !out) { set_last_error(kErrInvalid, "dsim_config_load: null argument"); return kErrInvalid; }
    std::string text;
    if (!read_file(path, text)) { set_last_error(kErrFile, "cannot read %s", path); return kErrFile; }
    CfgParser P(text);
    if (!P.settings("") || P.i < text.size()) {
        set_last_error(kErrFormat, "%s: config syntax error near byte %zu", path, P.i);
        return kErrFormat;
    }
    auto& kv = P.kv;
    auto has = [&](const char* k) { return kv.count(k) > 0; };
    auto f = [&](const char* k, float d) { return has(k) ? strtof(kv[k].c_str(), nullptr) : d; };
    auto u = [&](const char* k, uint32_t d) { return has(k) ? (uint32_t)strtoul(kv[k].c_str(), nullptr, 10) : d; };
    auto b = [&](const char* k, int d) {
        if (!has(k)) return d;
        const std::string& v = kv[k];
        return (v == "true" || v == "TRUE" || v == "True") ? 1 : (v == "false" || v == "FALSE" || v == "False") ? 0
                                                                                                              : atoi(v.c_str());
    };
    auto str = [&](const char* k) { return has(k) ? kv[k] : std::string(); };
    memset(out, 0, sizeof(*out));
    const bool d2 = has("sim.timestep") || has("fibers.file") || has("sim.gyromagneticRatio");
    out->dialect = d2 ? 2 : 3;
    out->stepsPerUpdate = u("app.stepsPerUpdate", 10);
    out->useGpu = b("app.useGpu", 1);   // both reference mains default to the GPU
    out->useDisplay = b("app.useDisplay", 0);
    out->writeOut = b("app.writeOut", 1);
    out->numSpins = u("sim.numSpins", 1000);
    out->gamma = f(d2 ? "sim.gyromagneticRatio" : "sim.gyroMagneticRatio", 42576.0f);
    out->timeStep = f(d2 ? "sim.timestep" : "sim.timeStep", 0.005f);
    out->extraAdc = f("sim.extraAdc", 2.1f);
    out->intraAdc = f("sim.intraAdc", 2.1f);
    out->myelinAdc = f("sim.myelinAdc", 0.1f);
    out->extraT2 = f("sim.extraT2", 80.0f);
    out->intraT2 = f("sim.intraT2", 80.0f);
    out->myelinT2 = f("sim.myelinT2", 7.5f);
    out->spaceScale = f("sim.spaceScale", d2 ? 20.0f : 60.0f);
    out->startBox = f("sim.startBox", 1.0f);
    out->innerRadiusFraction = f("fibers.innerRadiusFraction", 0.7f);
    out->fiberRadius = f("fibers.radiusMean", 1.0f);
    out->fiberSpace = f("fibers.spacingMean", 0.2f);
    out->crossFraction = f("fibers.crossFraction", 0.0f);
    if (d2) out->permeability = (float)pow(10.0, (double)f("sim.permeability", -4.0f));
    else out->permeability = f("sim.permeability", 0.0f);
    set_str(out->gradsFile, str("sim.gradsFile"));
    set_str(out->gradsStr, str("sim.gradsStr"));
    set_str(out->outFile, str("sim.outFile"));
    set_str(out->fiberFile, str(d2 ? "fibers.file" : "fibers.fiberFile"));
    return kOk;
}

int dsim_grads_parse_file(const char* path, float* rows, uint32_t cap, uint32_t* n) {
    if (!path || !n) { set_last_error(kErrInvalid, "dsim_grads_parse_file: null argument"); return kErrInvalid; }
    std::string text;
    if (!read_file(path, text)) { set_last_error(kErrFile, "cannot read %s", path); return kErrFile; }
    return parse_rows(text, rows, cap, n);
}

int dsim_grads_parse_string(const char* text, float* rows, uint32_t cap, uint32_t* n) {
    if (!text || !n) { set_last_error(kErrInvalid, "dsim_grads_parse_string: null argument"); return kErrInvalid; }
    return parse_rows(std::string(text), rows, cap, n);
}

int dsim_pgse_schedule(const float row[6], float timeStep, uint32_t spu, float* grad, uint32_t cap, uint32_t* nSteps) {
    if (!row || !nSteps || spu == 0 || !(timeStep > 0.0f)) { set_last_error(kErrInvalid, "dsim_pgse_schedule: bad argument"); return kErrInvalid; }
    const Sched s = schedule(row, timeStep, spu);
    if (s.nUpdates < 0) { set_last_error(kErrInvalid, "dsim_pgse_schedule: negative timing"); return kErrInvalid; }
    // update() reads the signal in the last branch of its chain: when the read
    // index coincides with an earlier branch (readout of zero updates) the
    // reference never reads this row's signal
    const int mIdx = s.bD + s.lD + s.ro;
    if (mIdx == 0 || mIdx == s.bD || mIdx == s.bD + s.lD) {
        set_last_error(kErrInvalid, "dsim_pgse_schedule: readout %g ms rounds to 0 updates; the reference's sequencer "
                       "never reads this row's signal", (double)row[2]);
        return kErrInvalid;
    }
    const uint64_t steps = (uint64_t)s.nUpdates * spu;
    *nSteps = (uint32_t)steps;
    if (!grad) return kOk;
    if (steps > cap) { set_last_error(kErrTooLarge, "dsim_pgse_schedule: %llu steps > capacity", (unsigned long long)steps); return kErrTooLarge; }
    const std::vector<float> w = update_signs(s);
    for (uint64_t t = 0; t < steps; t++) {
        const float g = w[(size_t)(t / spu)];
        grad[3 * t] = row[3] * g; grad[3 * t + 1] = row[4] * g; grad[3 * t + 2] = row[5] * g;
    }
    return kOk;
}

int dsim_tensor_fit(const float* rows, const double* signal, uint32_t nG, double tensor[9], double eigvecs[9],
                    float eigvals[3], float* md, float* fa, float* rd) {
    if (!rows || !signal || !tensor || !eigvecs || !eigvals) { set_last_error(kErrInvalid, "dsim_tensor_fit: null argument"); return kErrInvalid; }
    const double offset = 0.000001;
    double logB0 = 0.0;
    uint32_t nZero = 0;
    std::vector<double> M, adc;
    std::vector<double> logDw, bval;
    std::vector<double> dirs;
    for (uint32_t j = 0; j < nG; j++) {
        const double gx = rows[6 * j + 3], gy = rows[6 * j + 4], gz = rows[6 * j + 5];
        const double norm = sqrt(gx * gx + gy * gy + gz * gz);
        const double b = pow((2.0 * 3.1415926535 * 42576.0) * norm / 1000000000 * rows[6 * j + 0], 2) *
                         (rows[6 * j + 1] - rows[6 * j + 0] / 3.0);
        if (norm == 0) {
            logB0 += log(signal[j] + offset);
            nZero++;
        } else {
            dirs.push_back(gx / norm); dirs.push_back(gy / norm); dirs.push_back(gz / norm);
            logDw.push_back(log(signal[j] + offset));
            bval.push_back(b);
        }
    }
    if (nZero == 0 || logDw.size() < 6) {
        set_last_error(kErrInvalid, "dsim_tensor_fit: needs a zero gradient and 6 non-zero gradients");
        return kErrInvalid;
    }
    logB0 /= nZero;
    // least squares for {Dxx, Dyy, Dzz, Dxy, Dxz, Dyz}: rows [x^2, y^2, z^2, 2xy, 2xz, 2yz]
    double A[6][6] = {}, rhs[6] = {};
    for (size_t k = 0; k < logDw.size(); k++) {
        const double x = dirs[3 * k], y = dirs[3 * k + 1], z = dirs[3 * k + 2];
        const double r[6] = {x * x, y * y, z * z, 2 * x * y, 2 * x * z, 2 * y * z};
        const double a = -1.0 / bval[k] * (logDw[k] - logB0);
        for (int p = 0; p < 6; p++) {
            rhs[p] += r[p] * a;
            for (int q = 0; q < 6; q++) A[p][q] += r[p] * r[q];
        }
    }
    if (!solve6(A, rhs)) { set_last_error(kErrInvalid, "dsim_tensor_fit: gradient directions do not span a tensor"); return kErrInvalid; }
    double D[3][3] = {{rhs[0], rhs[3], rhs[4]}, {rhs[3], rhs[1], rhs[5]}, {rhs[4], rhs[5], rhs[2]}};
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) tensor[3 * r + c] = D[r][c];
    double V[3][3], d[3];
    jacobi3(D, V, d);
    int ord[3] = {0, 1, 2};
    for (int a = 0; a < 3; a++)
        for (int b2 = a + 1; b2 < 3; b2++)
            if (d[ord[b2]] < d[ord[a]]) std::swap(ord[a], ord[b2]);
    for (int k = 0; k < 3; k++) {
        eigvals[k] = (float)d[ord[k]];
        for (int r = 0; r < 3; r++) eigvecs[3 * r + k] = V[r][ord[k]];
    }
    const float m = (eigvals[0] + eigvals[1] + eigvals[2]) / 3.0f;
    if (md) *md = m;
    if (fa)
        *fa = (float)(sqrt(3.0 / 2.0) *
                      sqrt(pow(eigvals[0] - m, 2) + pow(eigvals[1] - m, 2) + pow(eigvals[2] - m, 2)) /
                      sqrt(pow(eigvals[0], 2) + pow(eigvals[1], 2) + pow(eigvals[2], 2)));
    if (rd) *rd = (eigvals[0] + eigvals[1]) / 2.0f;
    return kOk;
}

int dsim_write_results(const char* outFile, const dsim_config* cfgp, const float* rowsp, const double* signals,
                       uint32_t nG, double elapsed) {
    if (!outFile || !cfgp || (nG && (!rowsp || !signals))) {
        set_last_error(kErrInvalid, "dsim_write_results: null argument");
        return kErrInvalid;
    }
    const dsim_config& cfg = *cfgp;
    const std::vector<float> rows(rowsp, rowsp + 6 * (size_t)nG);
    const float dt = cfg.timeStep;
    // dSim3 keeps every signal in its float results table (gradientDataResults,
    // dSim3/src/diffusion.cpp:575-577), zeroed for the rows it never reads,
    // before it fits and prints them
    std::vector<double> sig32(5 * (size_t)nG);
    for (size_t k = 0; k < sig32.size(); k++) sig32[k] = std::isnan(signals[k]) ? 0.0 : (double)(float)signals[k];
    const double* signals64 = signals;
    if (cfg.dialect == 3) signals = sig32.data();
    FILE* f = fopen(outFile, "at");
    if (!f) { set_last_error(kErrFile, "cannot open %s", outFile); return kErrFile; }
    time_t now = time(nullptr);
    if (cfg.dialect == 3) {
        // dSim3/src/diffusion.cpp:666-728
        fprintf(f, "\n%% * * * %s", ctime(&now));
        fprintf(f, "if (exist('m','var')), m=m+1; else, m=1; end\n");
        fprintf(f, "s=0;\n");
        fprintf(f, "\n%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%% \n%% Input parameters \n%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%\n");
        fprintf(f, "numSpins(m) = %u;\n", cfg.numSpins);
        fprintf(f, "useGpu(m) = %d;\n", cfg.useGpu);
        fprintf(f, "fibersFile{m} = '%s';\n", cfg.fiberFile);
        fprintf(f, "useDisplay(m) = %d;\n", 0);
        fprintf(f, "stepsPerUpdate(m) = %i;\n", (int)cfg.stepsPerUpdate);
        fprintf(f, "gyroMagneticRatio(m) = %g;\n", cfg.gamma);
        fprintf(f, "timeStep(m) = %g;\n", cfg.timeStep);
        fprintf(f, "extraAdc(m) = %g;\n", cfg.extraAdc);
        fprintf(f, "intraAdc(m) = %g;\n", cfg.intraAdc);
        fprintf(f, "myelinAdc(m) = %g;\n", cfg.myelinAdc);
        fprintf(f, "spaceScale(m) = %g;\n", cfg.spaceScale);
        fprintf(f, "permeability(m) = %g;\n", cfg.permeability);
        fprintf(f, "\n\n%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%% \n%% Simulation data \n%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%%\n\n");
        fprintf(f, "%%The following variables give the diffusion tensor, eigenvector matrix, eigenvalues\n");
        fprintf(f, "%%(eigenvalue no. i corresponds to column no. i in the eigenvector matrix), mean diffusivity,\n");
        fprintf(f, "%%fractional anisotropy and radial diffusivity for the whole volume (index 1) and each\n");
        fprintf(f, "%%compartment (index 2 for compartment 0, index 3 for compartment 1, etc).\n");
        // the reference writes the fits of the total signal and compartments 0-2 as indices 1-4
        for (int ci = 0; ci < 4; ci++) {
            std::vector<double> sg(nG);
            for (uint32_t g = 0; g < nG; g++) sg[g] = signals[5 * (size_t)g + ci];
            double T[9] = {0}, E[9] = {0};
            float ev[3] = {0, 0, 0}, mdv = 0, fav = 0, rdv = 0;
            dsim_tensor_fit(rows.data(), sg.data(), nG, T, E, ev, &mdv, &fav, &rdv);
            fprintf(f, "tensor{m}{%u} = [%g, %g, %g; %g, %g, %g; %g, %g, %g];\n", ci + 1, T[0], T[1], T[2], T[3], T[4], T[5], T[6], T[7], T[8]);
            fprintf(f, "eigenvecs{m}{%u} = [%g, %g, %g; %g, %g, %g; %g, %g, %g];\n", ci + 1, E[0], E[1], E[2], E[3], E[4], E[5], E[6], E[7], E[8]);
            fprintf(f, "eigenvals{m}{%u} = [%g,%g,%g];\n", ci + 1, ev[0], ev[1], ev[2]);
            fprintf(f, "md{m}(%u) = %g;\n", ci + 1, mdv);
            fprintf(f, "fa{m}(%u) = %g;\n", ci + 1, fav);
            fprintf(f, "rd{m}(%u) = %g;\n", ci + 1, rdv);
        }
        fprintf(f, "%%The following variables give results for each gradient run.\n");
        fprintf(f, "%%mrSigTotal{m}(c,s) is the total signal after gradient run s during diffusion simulation no. m\n");
        fprintf(f, "%%mrSigCompartments{m}(c,s) is the contribution of compartment no. (c-2) to the \n");
        fprintf(f, "%%total signal after gradient run s during diffusion simulation no. m. c=1 represents all compartments. \n");
        for (uint32_t g = 0; g < nG; g++) {
            const float* r = &rows[6 * g];
            fprintf(f, "\ns=s+1;\n");
            fprintf(f, "delta{m}(s) = %g;\n", r[0]);
            fprintf(f, "Delta{m}(s) = %g;\n", r[1]);
            fprintf(f, "readOut{m}(s) = %g;\n", r[2]);
            fprintf(f, "dwGrads{m}(:,s) = [%g,%g,%g];\n\n", r[3], r[4], r[5]);
            fprintf(f, "mrSigTotal{m}(s) = %g;\n\n", signals[5 * (size_t)g]);
            for (int ci = 0; ci < 4; ci++)
                fprintf(f, "mrSigCompartments{m}(%u,s) = %g;\n", ci + 1, signals[5 * (size_t)g + 1 + ci]);
        }
    } else {
        // dSim2/src/diffusion.cpp:1756-1770 (header), 232-276 (per run, timing)
        fprintf(f, "\n%% * * * %s", ctime(&now));
        fprintf(f, "if(exist('m','var')), m=m+1; else, m=1; end\n");
        fprintf(f, "s=0;\n");
        fprintf(f, "radiusMean(m) = %g;\n", cfg.fiberRadius);
        fprintf(f, "radiusSpace(m) = %g;\n", cfg.fiberSpace);
        fprintf(f, "spaceScale(m) = %g;\n", cfg.spaceScale);
        fprintf(f, "numSpins(m) = %d;\n", (int)cfg.numSpins);
        fprintf(f, "crossFraction(m) = %g;\n", cfg.crossFraction);
        fprintf(f, "useGpu(m) = %d;\n", cfg.useGpu);
        fprintf(f, "fibersFile{m} = '%s';\n", cfg.fiberFile);
        double totalSteps = 0.0;
        for (uint32_t g = 0; g < nG; g++) {
            const float* r = &rows[6 * g];
            uint32_t steps = 0;
            const bool read = dsim_pgse_schedule(r, dt, cfg.stepsPerUpdate, nullptr, 0, &steps) == kOk;
            totalSteps += steps;
            fprintf(f, "s = s+1;\n");
            fprintf(f, "delta{m}(s) = %g;\n", r[0]);
            fprintf(f, "Delta{m}(s) = %g;\n", r[1]);
            fprintf(f, "readOut{m}(s) = %g;\n", r[2]);
            fprintf(f, "dwGrads{m}(:,s) = [%g;%g;%g];\n", r[3], r[4], r[5]);
            if (read) fprintf(f, "mrSig{m}(s) = %g;\n", signals64[5 * (size_t)g]);
        }
        fprintf(f, "%% Timing info:\n");
        fprintf(f, "stepsPerSec(m) = %g;\n", elapsed > 0 ? totalSteps / elapsed : 0.0);
        fprintf(f, "totalTime(m) = %g;\n", elapsed);
    }
    fclose(f);
    return kOk;
}

int dsim_simulate(const char* cfgPath, uint64_t seed, uint32_t flags, double* signals, uint32_t cap, uint32_t* nGout,
                  double* seconds) {
    dsim_config cfg;
    int rc = dsim_config_load(cfgPath, &cfg);
    if (rc) return rc;
    std::vector<float> rows;
    uint32_t nG = 0;
    if (cfg.gradsFile[0]) {
        const std::string gp = resolve(cfgPath, cfg.gradsFile);
        if ((rc = dsim_grads_parse_file(gp.c_str(), nullptr, 0, &nG))) return rc;
        rows.resize((size_t)nG * 6);
        if ((rc = dsim_grads_parse_file(gp.c_str(), rows.data(), nG, &nG))) return rc;
    } else if (cfg.gradsStr[0]) {
        if ((rc = dsim_grads_parse_string(cfg.gradsStr, nullptr, 0, &nG))) return rc;
        rows.resize((size_t)nG * 6);
        if ((rc = dsim_grads_parse_string(cfg.gradsStr, rows.data(), nG, &nG))) return rc;
    }
    if (nGout) *nGout = nG;
    if (!signals || cap < nG) { set_last_error(kErrTooLarge, "dsim_simulate: %u gradients > capacity %u", nG, cap); return kErrTooLarge; }
    const std::string fiberPath = resolve(cfgPath, cfg.fiberFile);
    std::string head;
    if (!read_file(fiberPath.c_str(), head)) { set_last_error(kErrFile, "cannot read fiber file %s", fiberPath.c_str()); return kErrFile; }
    size_t k0 = head.find_first_not_of(" \t\r\n");
    const bool mesh = k0 != std::string::npos && strchr("VTAMG", head[k0]) != nullptr;
    const uint32_t N = cfg.numSpins;
    const float ss = cfg.spaceScale, dt = cfg.timeStep;
    const float pc = 6.28318530717959f * cfg.gamma * dt;  // phaseConstant, SpinSystem::updateSpins
    const bool shared = (flags & DSIM_SIM_SHARED_WALK) != 0;
    double elapsed = 0.0;

    dsim_mesh* m = nullptr;
    dsim_cyl* c = nullptr;
    dsim_spins* s = nullptr;
    dsim_batch* b = nullptr;
    std::vector<float> fp;
    std::vector<uint32_t> cc, cubes;
    uint32_t geom[3] = {0, 0, 0};
    float L = 0.0f;
    // SpinSystem ctor sigma per compartment: sqrt(2 ADC / spaceScale^2 dt) (dSim3/src/spinSystem.cpp:52-56)
    const float sd3[4] = {sqrtf(2.0f * cfg.extraAdc / (ss * ss) * dt), sqrtf(2.0f * cfg.intraAdc / (ss * ss) * dt),
                          sqrtf(2.0f * cfg.myelinAdc / (ss * ss) * dt), sqrtf(2.0f * cfg.intraAdc / (ss * ss) * dt)};
    const float T23[4] = {cfg.extraT2, cfg.intraT2, cfg.myelinT2, cfg.intraT2};
    if (mesh) {
        if ((rc = dsim_mesh_load(fiberPath.c_str(), ss, 50, &m))) return rc;
    } else {
        if ((rc = dsim_cyl_load(fiberPath.c_str(), ss, &c))) return rc;
        dsim_cyl_info(c, geom, &L, nullptr, nullptr, nullptr);
        const size_t n3 = (size_t)geom[0] * geom[0] * geom[0];
        cc.resize(n3); cubes.resize(std::max<size_t>(1, n3 * geom[1])); fp.resize(std::max<size_t>(1, 4 * (size_t)geom[2]));
        dsim_cyl_info(c, geom, &L, cc.data(), cubes.data(), fp.data());
    }
    auto cleanup = [&]() {
        if (s) dsim_spins_free(s);
        if (b) dsim_batch_free(b);
        if (m) dsim_mesh_free(m);
        if (c) dsim_cyl_free(c);
    };
    const float box = mesh ? cfg.startBox : 1.0f;
    const double region = mesh ? 0.0 : 0.8;
    if (!shared) {
        if ((rc = dsim_spins_create(N, &s))) { cleanup(); return rc; }
        for (uint32_t g = 0; g < nG && !rc; g++) {
            uint32_t steps = 0;
            if (dsim_pgse_schedule(&rows[6 * g], dt, cfg.stepsPerUpdate, nullptr, 0, &steps)) {
                for (int q = 0; q < 5; q++) signals[5 * (size_t)g + q] = NAN;  // never read by the reference
                continue;
            }
            std::vector<float> gps(3 * (size_t)steps);
            dsim_pgse_schedule(&rows[6 * g], dt, cfg.stepsPerUpdate, gps.data(), steps, &steps);
            for (auto& v : gps) v = v * 1e-9f * ss;  // gradScaled (dSim3/src/spinSystem.cpp:1931)
            std::vector<float> pos = reset_positions(N, seed, g, box);
            std::vector<float> ones(N, 1.0f), zeros(N, 0.0f);
            const auto t0 = std::chrono::steady_clock::now();
            if (mesh) {
                std::vector<uint8_t> comp(N, 0);
                std::vector<uint16_t> fib(N, 0xFFFF);
                if ((rc = dsim_spins_set(s, pos.data(), ones.data(), zeros.data(), comp.data(), fib.data()))) break;
                if ((rc = dsim_mesh_compartments(m, s, seed ^ (0x9E3779B97F4A7C15ull * (g + 1)), box, nullptr))) break;
                dsim_mesh_params p;
                memset(&p, 0, sizeof(p));
                for (int k = 0; k < 4; k++) { p.stdDevs[k] = sd3[k]; p.T2[k] = T23[k]; }
                p.permeability = cfg.permeability;
                p.reflectionType = 1;
                p.spinRadius = 0.005f;
                p.deltaTime = dt;
                p.phaseConstant = pc;
                const float g0[3] = {0, 0, 0};
                rc = dsim_mesh_run(m, s, &p, g0, gps.data(), steps, seed + g, 0, nullptr, 0);
            } else {
                std::vector<uint32_t> imo, nearest;
                cyl_regions_host(pos, fp, cc, cubes, geom[0], geom[1], L, cfg.innerRadiusFraction, imo, nearest);
                if ((rc = dsim_spins_set_cyl(s, pos.data(), ones.data(), zeros.data(), imo.data(), nearest.data()))) break;
                dsim_cyl_params p;
                memset(&p, 0, sizeof(p));
                p.intraAdc = cfg.intraAdc; p.extraAdc = cfg.extraAdc; p.myelinAdc = cfg.myelinAdc;
                p.spaceScale = ss;
                p.T2fiber = cfg.intraT2; p.T2myelin = cfg.myelinT2; p.T2outside = cfg.extraT2;
                p.permeability = cfg.permeability;
                p.innerRadiusProportion = cfg.innerRadiusFraction;
                p.spinRadius = 0.005f;
                p.deltaTime = dt;
                p.phaseConstant = pc;
                const float g0[3] = {0, 0, 0};
                rc = dsim_cyl_run(c, s, &p, g0, gps.data(), steps, seed + g, 0, nullptr, 0);
            }
            double sums[15];
            if (!rc) rc = dsim_signal(s, region, sums);
            elapsed += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            for (int q = 0; q < 5; q++) signals[5 * (size_t)g + q] = sig_of(sums, q);
        }
    } else {
        // one walk per timing group; every gradient of the group from the moments
        std::vector<int> done(nG, 0);
        uint32_t group = 0;
        for (uint32_t g = 0; g < nG && !rc; g++) {
            if (done[g]) continue;
            std::vector<uint32_t> members;
            for (uint32_t h = g; h < nG; h++)
                if (!done[h] && rows[6 * h] == rows[6 * g] && rows[6 * h + 1] == rows[6 * g + 1] &&
                    rows[6 * h + 2] == rows[6 * g + 2]) {
                    members.push_back(h);
                    done[h] = 1;
                }
            const float unit[6] = {rows[6 * g], rows[6 * g + 1], rows[6 * g + 2], 1.0f, 0.0f, 0.0f};
            uint32_t steps = 0;
            if (dsim_pgse_schedule(unit, dt, cfg.stepsPerUpdate, nullptr, 0, &steps)) {
                for (uint32_t h : members)
                    for (int q = 0; q < 5; q++) signals[5 * (size_t)h + q] = NAN;  // never read by the reference
                continue;
            }
            std::vector<float> gps(3 * (size_t)steps), w(steps);
            dsim_pgse_schedule(unit, dt, cfg.stepsPerUpdate, gps.data(), steps, &steps);
            for (uint32_t t = 0; t < steps; t++) w[t] = gps[3 * (size_t)t];
            std::vector<float> pos = reset_positions(N, seed, group, box);
            std::vector<uint8_t> comp(N, 0);
            std::vector<uint32_t> fib(N, 0xFFFFFFFFu);
            if (mesh) {
                // compartments from a spin object, then the batch job
                dsim_spins* tmp = nullptr;
                std::vector<float> ones(N, 1.0f), zeros(N, 0.0f);
                std::vector<uint16_t> f16(N, 0xFFFF);
                if ((rc = dsim_spins_create(N, &tmp))) break;
                rc = dsim_spins_set(tmp, pos.data(), ones.data(), zeros.data(), comp.data(), f16.data());
                if (!rc) rc = dsim_mesh_compartments(m, tmp, seed ^ (0x9E3779B97F4A7C15ull * (group + 1)), box, nullptr);
                if (!rc) rc = dsim_spins_get(tmp, pos.data(), nullptr, nullptr, comp.data(), f16.data());
                dsim_spins_free(tmp);
                if (rc) break;
                for (uint32_t i = 0; i < N; i++) fib[i] = f16[i];
            } else {
                std::vector<uint32_t> imo, nearest;
                cyl_regions_host(pos, fp, cc, cubes, geom[0], geom[1], L, cfg.innerRadiusFraction, imo, nearest);
                for (uint32_t i = 0; i < N; i++) { comp[i] = (uint8_t)imo[i]; fib[i] = nearest[i]; }
            }
            if (b) { dsim_batch_free(b); b = nullptr; }
            if ((rc = dsim_batch_create((N + 31) & ~31u, 1, &b))) break;
            uint32_t sub = 0;
            rc = mesh ? dsim_batch_add_mesh(b, m, &sub) : dsim_batch_add_cyl(b, c, &sub);
            if (rc) break;
            dsim_job_desc d;
            memset(&d, 0, sizeof(d));
            d.substrate = sub; d.nSpins = N; d.steps = steps; d.deltaTime = dt;
            if (mesh) {
                for (int k = 0; k < 4; k++) { d.stepSd[k] = sd3[k]; d.T2[k] = T23[k]; }
            } else {
                const float s2 = ss * ss;
                d.stepSd[0] = sqrtf(2.0f * (cfg.intraAdc / s2) * dt);
                d.stepSd[1] = sqrtf(2.0f * (cfg.myelinAdc / s2) * dt);
                d.stepSd[2] = sqrtf(2.0f * (cfg.extraAdc / s2) * dt);
                d.T2[0] = cfg.intraT2; d.T2[1] = cfg.myelinT2; d.T2[2] = cfg.extraT2;
            }
            d.permeability = cfg.permeability;
            d.reflectionType = 1;
            d.spinRadius = 0.005f;
            d.innerRadiusProportion = cfg.innerRadiusFraction;
            d.phaseConstant = pc;
            d.waveform = DSIM_WAVE_TABLE;
            d.table = w.data();
            d.seed = seed + group;
            uint32_t job = 0;
            const auto t0 = std::chrono::steady_clock::now();
            if ((rc = dsim_batch_submit(b, &d, pos.data(), comp.data(), fib.data(), &job))) break;
            if ((rc = dsim_batch_run(b))) break;
            std::vector<float> gs(3 * members.size());
            for (size_t q = 0; q < members.size(); q++)
                for (int k = 0; k < 3; k++) gs[3 * q + k] = rows[6 * members[q] + 3 + k] * 1e-9f * ss;
            std::vector<double> out(15 * members.size());
            rc = dsim_batch_signal_region(b, job, gs.data(), (uint32_t)members.size(), region, out.data());
            elapsed += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            for (size_t q = 0; q < members.size() && !rc; q++)
                for (int k = 0; k < 5; k++) signals[5 * (size_t)members[q] + k] = sig_of(&out[15 * q], k);
            group++;
        }
    }
    if (seconds) *seconds = elapsed;
    cleanup();
    if (rc) return rc;
    if ((flags & DSIM_SIM_WRITE_OUT) && cfg.outFile[0] && (cfg.dialect == 2 || cfg.writeOut))
        return dsim_write_results(cfg.outFile, &cfg, rows.data(), signals, nG, elapsed);
    return kOk;
}

}  // extern "C"
