"""numpy front end of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker.  The GPU engine never imports it.

The C library restates rfdougherty/dSim's CPU hot path (see oracle.h for the
function-by-function map to dSim3/src/spinKernelCpu.cpp, dSim3/src/spinSystem.cpp,
dSim2/src/spinKernelCpu.cpp and dSim2/src/spinSystem.cpp).
"""
import ctypes as C
import os
import struct

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
SOURCES = ["oracle_dsim3.c", "oracle_dsim2.c"]


def build(force=False):
    """Compile liboracle.so with the flags that keep float rounding identical
    to the reference's x86-64 build (no FMA contraction)."""
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    deps = srcs + [os.path.join(HERE, "oracle.h"), os.path.join(HERE, "dsim3_step.inc")]
    if not force and os.path.exists(LIB_PATH):
        t = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB_PATH
    import subprocess
    cc = os.environ.get("CC", "gcc")
    cmd = [cc, "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
           "-o", LIB_PATH + ".tmp"] + srcs + ["-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


_f = np.ctypeslib.ndpointer
P_F32 = _f(np.float32, flags="C_CONTIGUOUS")
P_F64 = _f(np.float64, flags="C_CONTIGUOUS")
P_U32 = _f(np.uint32, flags="C_CONTIGUOUS")
P_U16 = _f(np.uint16, flags="C_CONTIGUOUS")
P_U8 = _f(np.uint8, flags="C_CONTIGUOUS")


class Params3(C.Structure):
    _fields_ = [("stdDevs", C.c_float * 4), ("T2", C.c_float * 4), ("permeability", C.c_float),
                ("reflectionType", C.c_uint32), ("spinRadius", C.c_float), ("deltaTime", C.c_float),
                ("numCubes", C.c_uint32), ("maxTrianglesPerCube", C.c_uint32),
                ("cubeLength", C.c_float), ("maxSubsegments", C.c_uint32)]


class Params2(C.Structure):
    _fields_ = [("intraAdcScaled", C.c_float), ("extraAdcScaled", C.c_float),
                ("myelinAdcScaled", C.c_float), ("T2fiber", C.c_float), ("T2myelin", C.c_float),
                ("T2outside", C.c_float), ("permeability", C.c_float),
                ("innerRadiusProportion", C.c_float), ("spinRadius", C.c_float),
                ("deltaTime", C.c_float), ("numCubes", C.c_uint32), ("maxFibersPerCube", C.c_uint32),
                ("cubeLength", C.c_float)]


def _opt(ptrtype):
    """ndpointer that also accepts None."""
    class _Opt(ptrtype):
        @classmethod
        def from_param(cls, obj):
            if obj is None:
                return None
            return ptrtype.from_param(obj)
    return _Opt


def _declare(L):
    L.or_philox4x32_10.argtypes = [P_U32, P_U32, P_U32]
    L.or_myrandn.argtypes = [P_U32, P_F32]
    L.or3_mesh_count.argtypes = [C.c_char_p, P_U32]
    L.or3_mesh_count.restype = C.c_int
    L.or3_mesh_fill.argtypes = [C.c_char_p, C.c_float, P_U32, P_F32, P_U32, P_U32, P_F32, P_F32]
    L.or3_populate_count.argtypes = [C.c_uint32, P_F32, P_U32, C.c_uint32, P_U32]
    L.or3_populate_count.restype = C.c_uint32
    L.or3_populate_fill.argtypes = [C.c_uint32, P_F32, P_U32, C.c_uint32, C.c_uint32, P_U32, P_U32]
    L.or3_integrate.argtypes = [C.POINTER(Params3), C.c_uint32, P_F32, P_U32, P_F32, P_F32, P_U8,
                                P_U16, P_F32, P_F32, P_U32, P_U32, P_U32, C.c_float, C.c_float,
                                C.c_float, C.c_float, C.c_uint32, _opt(P_F32), _opt(P_F32),
                                _opt(P_U32)]
    L.or3_integrate.restype = C.c_uint32
    L.or3_integrate_mt.argtypes = [C.POINTER(Params3), C.c_uint32, P_F32, P_U32, P_F32, P_F32, P_U8,
                                   P_U16, P_F32, P_F32, P_U32, P_U32, P_U32, C.c_float, C.c_float,
                                   C.c_float, C.c_float, C.c_uint32, C.c_int]
    L.or3_integrate_mt.restype = C.c_uint32
    L.or3_integrate_f64.argtypes = [C.POINTER(Params3), C.c_uint32, P_F64, P_F64, P_F64, P_U8,
                                    P_U16, C.c_uint32, P_F64, P_U32, P_U32, P_U32, P_U32, P_F64,
                                    C.c_double, C.c_uint32, P_F32, _opt(P_U32)]
    L.or3_integrate_f64.restype = C.c_uint32
    L.or3_integrate_f64_moments.argtypes = [C.POINTER(Params3), C.c_uint32, P_F64, P_F64, P_U8, P_U16,
                                            C.c_uint32, P_F64, P_U32, P_U32, P_U32, P_U32, C.c_uint32,
                                            P_F64, C.c_uint32, P_F32, P_F64, _opt(P_U32), C.c_int]
    L.or3_integrate_f64_moments.restype = C.c_uint32
    L.or3_integrate_multi.argtypes = [C.POINTER(Params3), C.c_uint32, P_F32, P_U32, P_F32, P_U8, P_U16,
                                      P_F32, P_F32, P_U32, P_U32, P_U32, C.c_uint32, P_F32, P_F32,
                                      C.c_float, C.c_uint32, _opt(P_F32), P_F32, _opt(P_U32), C.c_int]
    L.or3_integrate_multi.restype = C.c_uint32
    L.or2_integrate_multi.argtypes = [C.POINTER(Params2), C.c_uint32, P_F32, P_U32, P_F32, P_F32, P_U32,
                                      P_U32, C.c_uint32, P_F32, P_F32, C.c_float, C.c_uint32, _opt(P_F32),
                                      P_F32, _opt(P_U32), C.c_int]
    L.or2_integrate_f64_multi.argtypes = [C.POINTER(Params2), C.c_uint32, P_F64, P_F64, P_U32, P_U32, P_F32,
                                          P_U32, P_U32, C.c_uint32, P_F64, P_F64, C.c_double, C.c_uint32, P_F32,
                                          P_F64, C.c_int]
    L.or3_signal.argtypes = [C.c_uint32, P_F32, P_F32, P_U8, P_F64]
    L.or2_load_fibers.argtypes = [C.c_char_p, C.c_float, _opt(P_F32), C.POINTER(C.c_float)]
    L.or2_load_fibers.restype = C.c_int
    L.or2_build_grid.argtypes = [C.c_uint32, P_F32, C.c_float, P_U32, C.POINTER(C.c_float),
                                 _opt(P_U32), _opt(P_U32)]
    L.or2_build_grid.restype = C.c_int
    L.or2_find_nearest.argtypes = [C.c_uint32, P_F32, P_F32, C.c_uint32, C.c_float, C.c_uint32,
                                   P_U32, P_U32, C.c_float, P_U32, P_U32]
    L.or2_integrate.argtypes = [C.POINTER(Params2), C.c_uint32, P_F32, P_U32, P_F32, P_F32, P_U32,
                                P_U32, C.c_float, C.c_float, C.c_float, C.c_float, C.c_uint32,
                                _opt(P_F32), _opt(P_F32), _opt(P_U32)]
    L.or2_signal.argtypes = [C.c_uint32, P_F32, P_F32]
    L.or2_signal.restype = C.c_double


# --------------------------------------------------------------------------
def philox(ctr, key):
    out = np.zeros(4, np.uint32)
    lib().or_philox4x32_10(np.asarray(ctr, np.uint32), np.asarray(key, np.uint32), out)
    return out


def myrandn(seed2):
    s = np.array(seed2, np.uint32)
    out = np.zeros(4, np.float32)
    lib().or_myrandn(s, out)
    return out, s


class Mesh:
    """The reference's mesh arrays after SpinSystem::initFibers."""

    def __init__(self, path, spaceScale):
        L = lib()
        counts = np.zeros(7, np.uint32)
        rc = L.or3_mesh_count(path.encode(), counts)
        if rc != 0:
            raise ValueError("mesh file %s rejected (%d)" % (path, rc))
        self.counts = counts
        nV, nT = int(counts[0]), int(counts[1])
        self.vertices = np.zeros(3 * nV, np.float32)
        self.trgls = np.zeros(3 * nT, np.uint32)
        self.triInfo = np.zeros(3 * nT, np.uint32)
        self.helpers = np.zeros(12 * nT, np.float32)
        self.maxabs = np.zeros(3, np.float32)
        L.or3_mesh_fill(path.encode(), spaceScale, counts, self.vertices, self.trgls,
                        self.triInfo, self.helpers, self.maxabs)
        self.nV, self.nT = nV, nT


def populate_cubes(vertices, trgls, numCubes=50):
    """populateCubes: dense [cell][maxTrianglesPerCube] lists + counters."""
    L = lib()
    nT = len(trgls) // 3
    cc = np.zeros(numCubes ** 3, np.uint32)
    maxtpc = L.or3_populate_count(nT, vertices, trgls, numCubes, cc)
    tic = np.zeros(max(1, numCubes ** 3 * maxtpc), np.uint32)
    L.or3_populate_fill(nT, vertices, trgls, numCubes, maxtpc, cc, tic)
    return cc, tic, int(maxtpc)


def params3(stdDevs, T2, permeability, deltaTime, numCubes, maxTPC, reflectionType=1,
            spinRadius=0.005, maxSubsegments=0):
    p = Params3()
    p.stdDevs[:] = [float(x) for x in stdDevs]
    p.T2[:] = [float(x) for x in T2]
    p.permeability = permeability
    p.reflectionType = reflectionType
    p.spinRadius = spinRadius
    p.deltaTime = deltaTime
    p.numCubes = numCubes
    p.maxTrianglesPerCube = maxTPC
    p.cubeLength = np.float32(2.0) / np.float32(numCubes)
    p.maxSubsegments = maxSubsegments
    return p


def integrate3(p, pos, seed, mag, phase, comp, fiber, vertices, helpers, triInfo, cc, tic,
               g, phaseConstant, iterations, draws=None, record_draws=False, counts=None):
    """In-place dSim3 step x iterations.  Returns (capped, drawsOut)."""
    N = len(mag)
    dout = np.zeros((iterations, N, 4), np.float32) if record_draws else None
    d = None if draws is None else np.ascontiguousarray(draws, np.float32).reshape(-1)
    capped = lib().or3_integrate(C.byref(p), N, pos, seed, mag, phase, comp, fiber, vertices,
                                 helpers, triInfo, cc, tic, float(g[0]), float(g[1]), float(g[2]),
                                 float(phaseConstant), iterations, d,
                                 None if dout is None else dout.reshape(-1), counts)
    return capped, dout


def integrate3_multi(p, pos, seed, mag, comp, fiber, vertices, helpers, triInfo, cc, tic, grads, wave,
                     phaseConstant, draws=None, counts=None, nthreads=None):
    """One dSim3 walk (MWC draws from `seed`, or replay `draws`) giving the
    reference's phase for every gradient run: returns phases [N][nG].  pos,
    seed, mag, comp, fiber are updated in place; wave[t] scales grads at step t."""
    N = len(mag)
    g = np.ascontiguousarray(grads, np.float32).reshape(-1, 3)
    w = np.ascontiguousarray(wave, np.float32)
    ph = np.zeros(N * len(g), np.float32)
    d = None if draws is None else np.ascontiguousarray(draws, np.float32).reshape(-1)
    capped = lib().or3_integrate_multi(C.byref(p), N, pos, seed, mag, comp, fiber, vertices, helpers, triInfo, cc,
                                       tic, len(g), g.reshape(-1), w, float(phaseConstant), len(w), d, ph, counts,
                                       int(nthreads or os.cpu_count() or 1))
    return capped, ph.reshape(N, len(g))


def integrate2_multi(p, pos4, seed4, params5, fiberPos, cc, cubes, grads, wave, phaseConstant, draws=None,
                     counts=None, nthreads=None):
    """One dSim2 walk giving the reference's phase for every gradient run:
    returns phases [N][nG]; pos4, seed4, params5 are updated in place."""
    N = len(pos4) // 4
    g = np.ascontiguousarray(grads, np.float32).reshape(-1, 3)
    w = np.ascontiguousarray(wave, np.float32)
    ph = np.zeros(N * len(g), np.float32)
    d = None if draws is None else np.ascontiguousarray(draws, np.float32).reshape(-1)
    lib().or2_integrate_multi(C.byref(p), N, pos4, seed4, params5, fiberPos, cc, cubes, len(g), g.reshape(-1), w,
                              float(phaseConstant), len(w), d, ph, counts, int(nthreads or os.cpu_count() or 1))
    return ph.reshape(N, len(g))


def integrate2_f64_multi(p, pos3, mag, imo, nearest, fiberPos, cc, cubes, grads, wave, phaseConstant, draws,
                        nthreads=None):
    """FP64 cylinder walk on replay draws [iters][N][4]; returns phases [N][nG]
    (double).  pos3 (float64 [N*3]), mag (float64), imo, nearest (uint32) are
    updated in place."""
    N = len(mag)
    g = np.ascontiguousarray(grads, np.float64).reshape(-1, 3)
    w = np.ascontiguousarray(wave, np.float64)
    ph = np.zeros(N * len(g), np.float64)
    d = np.ascontiguousarray(draws, np.float32).reshape(-1)
    assert len(d) == 4 * N * len(w)
    lib().or2_integrate_f64_multi(C.byref(p), N, pos3, mag, imo, nearest, fiberPos, cc, cubes, len(g), g.reshape(-1),
                                  w, float(phaseConstant), len(w), d, ph, int(nthreads or os.cpu_count() or 1))
    return ph.reshape(N, len(g))


def signal3(mag, phase, comp):
    out = np.zeros(5, np.float64)
    lib().or3_signal(len(mag), mag, phase, comp, out)
    return out


# ---- cylinders ----------------------------------------------------------
def load_fibers2(path, spaceScale):
    L = lib()
    n = L.or2_load_fibers(path.encode(), spaceScale, None, None)
    if n < 0:
        raise ValueError("cannot open %s" % path)
    fp = np.zeros(4 * max(n, 1), np.float32)
    mr = C.c_float(0)
    L.or2_load_fibers(path.encode(), spaceScale, fp, C.byref(mr))
    return fp[:4 * n], float(mr.value)


def build_grid2(fiberPos, maxR):
    L = lib()
    nF = len(fiberPos) // 4
    geom = np.zeros(2, np.uint32)
    cl = C.c_float(0)
    L.or2_build_grid(nF, fiberPos, maxR, geom, C.byref(cl), None, None)
    n, maxfpc = int(geom[0]), int(geom[1])
    cc = np.zeros(n ** 3, np.uint32)
    cubes = np.zeros(max(1, n ** 3 * maxfpc), np.uint32)
    rc = L.or2_build_grid(nF, fiberPos, maxR, geom, C.byref(cl), cc, cubes)
    if rc != 0:
        raise ValueError("cylinder grid overflow (maxFibersPerCube=%d)" % maxfpc)
    return cc, cubes, n, maxfpc, np.float32(cl.value)


# --------------------------------------------------------------------------
def read_dump(path):
    """Reader for the reference harness dumps (oracle/refharness/dump.h)."""
    out = {}
    with open(path, "rb") as fh:
        data = fh.read()
    off = 0
    while off < len(data):
        name = data[off:off + 32].split(b"\0")[0].decode()
        dt = data[off + 32:off + 40].split(b"\0")[0].decode()
        (cnt,) = struct.unpack("<Q", data[off + 40:off + 48])
        off += 48
        dtype = np.dtype("<" + dt)
        nb = cnt * dtype.itemsize
        out[name] = np.frombuffer(data[off:off + nb], dtype).copy()
        off += nb
    return out


def spin_fields(raw):
    """Split raw spinData records (12 B: f32 mag, f32 phase, u8 comp, pad, u16 fiber)."""
    rec = np.frombuffer(raw.tobytes(), np.dtype([("mag", "<f4"), ("phase", "<f4"), ("comp", "u1"),
                                                 ("pad", "u1"), ("fiber", "<u2")]))
    return (rec["mag"].copy(), rec["phase"].copy(), rec["comp"].copy(), rec["fiber"].copy())


def integrate3_f64_moments(p, pos, mag, comp, fiber, vertices, trgls, triInfo, cc, tic, waves, draws,
                           counts=None, nthreads=1):
    """FP64 walk (the precision oracle) recording M_k = sum_t w_k(t) pos(t)
    for each waveform row of `waves` [nWaves][iterations].  pos, mag (float64)
    and comp, fiber are updated in place.  Returns (capped, moments[N][nWaves][3])."""
    L = lib()
    N = len(mag)
    waves = np.ascontiguousarray(waves, np.float64).reshape(-1, np.shape(waves)[-1])
    nW, iters = waves.shape
    mom = np.zeros(N * nW * 3, np.float64)
    v64 = np.ascontiguousarray(vertices, np.float64)
    capped = L.or3_integrate_f64_moments(C.byref(p), N, pos, mag, comp, fiber, len(trgls) // 3, v64,
                                         np.ascontiguousarray(trgls, np.uint32),
                                         np.ascontiguousarray(triInfo, np.uint32), cc,
                                         np.ascontiguousarray(tic, np.uint32), nW, waves.reshape(-1), iters,
                                         np.ascontiguousarray(draws, np.float32).reshape(-1), mom, counts,
                                         int(nthreads))
    return capped, mom.reshape(N, nW, 3)


# ---- the reference's driver around the path (restated in Python) -------------
def sequencer_runs(rows, timeStep, stepsPerUpdate):
    """dSim3/src/diffusion.cpp:522-737 (update()) replayed as a state machine:
    the gradient passed to every updateSpins call of each run, from the call
    that resets the spins to the one before the signal is read.  Returns a list
    of arrays [updates, 3] (mT/m), one per gradient row, or None for a row
    whose signal the reference never reads (the read branch is reached only
    when no earlier branch of the same update index matches)."""
    f32 = np.float32
    rows = np.asarray(rows, f32).reshape(-1, 6)
    curNumUpdates, nUpdates = 0, -1
    lD = bD = ro = 0
    curG = np.zeros(3, f32)
    g = np.zeros(3, f32)
    idx, done = 0, False
    runs, cur = [None] * len(rows), None
    while not done:
        measured = False
        if curNumUpdates <= nUpdates:
            if curNumUpdates == 0:
                cur = []
                g = curG.copy()
            elif curNumUpdates == lD and curNumUpdates < bD:
                g = np.zeros(3, f32)
            elif curNumUpdates == bD:
                g = curG * f32(-1.0)
            elif curNumUpdates == bD + lD:
                g = np.zeros(3, f32)
            elif curNumUpdates == bD + lD + ro:
                runs[idx - 1] = np.array(cur, f32).reshape(-1, 3)
                measured = True
            curNumUpdates += 1
        else:
            curNumUpdates = 0
            if idx >= len(rows):
                done = True
                continue
            r = rows[idx]
            idx += 1
            curG = r[3:6].copy()
            per = f32(timeStep) * f32(stepsPerUpdate)
            lD = int(float(r[0] / per) + 0.5)
            bD = int(float(r[1] / per) + 0.5)
            ro = int(float(r[2] / per) + 0.5)
            nUpdates = bD + lD + ro
            continue
        if cur is not None and not measured:
            cur.append(g.copy())          # updateSpins(timeStep, stepsPerUpdate) with gradient g
    return runs


def tensor_fit_reference(rows, signal):
    """computeTensor, dSim3/src/diffusion.cpp:286-511, restated with numpy:
    ADC per non-zero gradient, rows [x^2, y^2, z^2, 2xy, 2xz, 2yz] rounded to
    1e-6, pseudo-inverse from an SVD whose factors are rounded to 1e-6, then
    the eigen-decomposition (ascending) and md, fa, rd as float32."""
    rows = np.asarray(rows, np.float64).reshape(-1, 6)
    sig = np.asarray(signal, np.float64)
    rnd = lambda a: np.floor(a * 1000000.0 + 0.5) / 1000000.0
    norm = np.sqrt((rows[:, 3:6] ** 2).sum(1))
    b = ((2.0 * 3.1415926535 * 42576.0) * norm / 1000000000 * rows[:, 0]) ** 2 * (rows[:, 1] - rows[:, 0] / 3.0)
    zero = norm == 0
    logB0 = np.log(sig[zero] + 1e-6).mean()
    nz = ~zero
    adc = -1.0 / b[nz] * (np.log(sig[nz] + 1e-6) - logB0)
    d = rows[nz, 3:6] / norm[nz, None]
    M = rnd(np.stack([d[:, 0] ** 2, d[:, 1] ** 2, d[:, 2] ** 2, 2 * d[:, 0] * d[:, 1], 2 * d[:, 0] * d[:, 2],
                      2 * d[:, 1] * d[:, 2]], 1))
    U, S, Vt = np.linalg.svd(M, full_matrices=False)
    S, U, V = rnd(S), rnd(U), rnd(Vt.T)
    Sinv = np.where(S == 0, 0.0, 1.0 / np.where(S == 0, 1.0, S))
    Minv = rnd(V @ np.diag(Sinv) @ U.T)
    c = Minv @ adc
    D = np.array([[c[0], c[3], c[4]], [c[3], c[1], c[5]], [c[4], c[5], c[2]]])
    w, _ = np.linalg.eigh(D)
    lam = w.astype(np.float32)
    md = np.float32((lam[0] + lam[1] + lam[2]) / np.float32(3.0))
    fa = np.float32(np.sqrt(1.5) * np.sqrt(((lam.astype(np.float64) - md) ** 2).sum()) /
                    np.sqrt((lam.astype(np.float64) ** 2).sum()))
    rd = np.float32((lam[0] + lam[1]) / np.float32(2.0))
    return D, lam, md, fa, rd
