"""Python front end of the native engine (include/dsim.h).

MeshSystem and CylinderSystem hold a device-resident substrate and spin state
and mirror the calls of the reference's SpinSystem (dSim3/src/spinSystem.h:143-310,
dSim2/src/spinSystem.h:134-222): set the gradient, updateSpins(dt, iterations),
getMrSignal().  Unit conversions follow the reference exactly (float32
arithmetic in the same order) so that parameters match bit for bit.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, native

F = np.float32
TWOPI = F(6.28318530717959)  # dSim3/src/spinSystem.cpp:20


def std_devs(extraAdc, intraAdc, myelinAdc, spaceScale, deltaTime):
    """Per-compartment step sigma, SpinSystem ctor dSim3/src/spinSystem.cpp:52-56:
    sqrt(2*ADC/(spaceScale^2)*dt) for compartments 0 extra, 1 intra, 2 myelin, 3 glia(intra)."""
    ss = F(spaceScale)
    dt = F(deltaTime)
    out = []
    for adc in (extraAdc, intraAdc, myelinAdc, intraAdc):
        out.append(np.sqrt(F(2) * F(adc) / (ss * ss) * dt))
    return np.array(out, F)


def grad_scaled(G, spaceScale):
    """gradScaled = G[mT/m] * 1e-9f * spaceScale (dSim3/src/spinSystem.cpp:1931)."""
    g = np.asarray(G, F)
    return (g * F(1e-9)) * F(spaceScale)


def phase_constant(gamma, deltaTime):
    """2*pi*gamma*dt (dSim3/src/spinSystem.cpp:1938); gamma in kHz/T, dt in ms."""
    return TWOPI * F(gamma) * F(deltaTime)


class DeviceInfo:
    def __init__(self):
        name = C.create_string_buffer(256)
        sm = C.c_int(0)
        mem = C.c_size_t(0)
        check(native().dsim_device_info(name, 256, C.byref(sm), C.byref(mem)))
        self.name = name.value.decode()
        self.sm_count = sm.value
        self.total_mem = mem.value


class Spins:
    """Device-resident spin state with its own CUDA stream."""

    def __init__(self, N):
        self.N = int(N)
        h = C.c_void_p()
        check(native().dsim_spins_create(self.N, C.byref(h)))
        self.h = h

    def free(self):
        if self.h:
            native().dsim_spins_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def set(self, pos, mag=None, phase=None, comp=None, fiber=None):
        c = lambda a, t: None if a is None else np.ascontiguousarray(a, t)
        check(native().dsim_spins_set(self.h, c(pos, F).reshape(-1) if pos is not None else None,
                                      c(mag, F), c(phase, F), c(comp, np.uint8), c(fiber, np.uint16)))

    def get(self):
        N = self.N
        pos = np.zeros(3 * N, F); mag = np.zeros(N, F); ph = np.zeros(N, F)
        comp = np.zeros(N, np.uint8); fib = np.zeros(N, np.uint16)
        check(native().dsim_spins_get(self.h, pos, mag, ph, comp, fib))
        return pos, mag, ph, comp, fib

    def set_cyl(self, pos, mag=None, phase=None, imo=None, nearest=None):
        c = lambda a, t: None if a is None else np.ascontiguousarray(a, t)
        check(native().dsim_spins_set_cyl(self.h, c(pos, F).reshape(-1), c(mag, F), c(phase, F),
                                          c(imo, np.uint32), c(nearest, np.uint32)))

    def get_cyl(self):
        N = self.N
        pos = np.zeros(3 * N, F); mag = np.zeros(N, F); ph = np.zeros(N, F)
        imo = np.zeros(N, np.uint32); near = np.zeros(N, np.uint32)
        check(native().dsim_spins_get_cyl(self.h, pos, mag, ph, imo, near))
        return pos, mag, ph, imo, near

    def counts(self, reset=False):
        out = np.zeros(2 * self.N, np.uint32)
        check(native().dsim_spins_counts(self.h, out, 1 if reset else 0))
        return out.reshape(-1, 2)

    def set_sort_interval(self, steps):
        check(native().dsim_spins_set_sort_interval(self.h, int(steps)))

    def scanned(self, reset=False):
        out = np.zeros(self.N, np.uint32)
        check(native().dsim_spins_scanned(self.h, out, 1 if reset else 0))
        return out

    def status(self, reset=True):
        v = C.c_uint32(0)
        check(native().dsim_spins_status(self.h, C.byref(v), 1 if reset else 0))
        return v.value

    def signal(self, region=0.0):
        """FP64 sums per (all, compartment 0..3): array (5, 3) of X, Y, n."""
        out = np.zeros(15, np.float64)
        check(native().dsim_signal(self.h, float(region), out))
        return out.reshape(5, 3)

    def set_spin_base(self, base):
        """Global index of spin 0 in the random stream (replica shards)."""
        check(native().dsim_spins_set_spin_base(self.h, int(base)))

    def launches(self, reset=False):
        """Kernels launched by mesh/cylinder runs on this object."""
        n = C.c_uint64()
        check(native().dsim_spins_launches(self.h, C.byref(n), int(reset)))
        return n.value

    def sync(self):
        check(native().dsim_sync(self.h))

    def timer_start(self):
        check(native().dsim_timer_start(self.h))

    def timer_stop(self):
        ms = C.c_float(0)
        check(native().dsim_timer_stop(self.h, C.byref(ms)))
        return ms.value

    def flush_l2(self, nbytes=512 << 20):
        check(native().dsim_flush_l2(self.h, int(nbytes)))

    @property
    def nbytes(self):
        return int(native().dsim_spins_bytes(self.h))


def signal_from_sums(sums):
    """S = |X + iY| / n per row (0 when n = 0), as getMrSignal does."""
    s = np.asarray(sums, np.float64).reshape(-1, 3)
    out = np.zeros(len(s))
    nz = s[:, 2] > 0
    out[nz] = np.sqrt(s[nz, 0] ** 2 + s[nz, 1] ** 2) / s[nz, 2]
    return out


class Mesh:
    """Triangle-mesh substrate on the device with its GPU-built grid."""

    def __init__(self, handle):
        self.h = handle
        info = np.zeros(8, np.uint64)
        check(native().dsim_mesh_info(self.h, info))
        (self.nV, self.nT, self.nFibers, self.numCubes, self.entries, self.max_per_cell,
         self.nbytes, self.nonempty) = [int(x) for x in info]

    @classmethod
    def load(cls, path, spaceScale, numCubes=50):
        h = C.c_void_p()
        check(native().dsim_mesh_load(str(path).encode(), float(spaceScale), int(numCubes), C.byref(h)))
        return cls(h)

    @classmethod
    def from_arrays(cls, vertices_um, trgls, membrane, fiber, spaceScale, numCubes=50):
        v = np.ascontiguousarray(vertices_um, F).reshape(-1)
        t = np.ascontiguousarray(trgls, np.uint32).reshape(-1)
        m = None if membrane is None else np.ascontiguousarray(membrane, np.uint32)
        f = None if fiber is None else np.ascontiguousarray(fiber, np.uint32)
        h = C.c_void_p()
        check(native().dsim_mesh_create(v, len(v) // 3, t, m, f, len(t) // 3, float(spaceScale),
                                        int(numCubes), C.byref(h)))
        return cls(h)

    def set_accel(self, cells_per_axis):
        check(native().dsim_mesh_set_accel(self.h, int(cells_per_axis)))

    def set_records(self, nbytes):
        check(native().dsim_mesh_set_records(self.h, int(nbytes)))

    def compartments(self, spins, seed=1, start_box=1.0):
        """Assign every spin's compartment and fiber from its position (ray
        parity, as findSpinsInFibers); returns the number of spins moved."""
        moved = C.c_uint32()
        check(native().dsim_mesh_compartments(self.h, spins.h, int(seed), float(start_box), C.byref(moved)))
        return moved.value

    def set_kernel(self, variant):
        check(native().dsim_mesh_set_kernel(self.h, int(variant)))

    def accel_info(self):
        info = np.zeros(3, np.uint64)
        check(native().dsim_mesh_accel_info(self.h, info))
        return dict(cells=int(info[0]), entries=int(info[1]), nbytes=int(info[2]))

    def grid(self):
        n3 = self.numCubes ** 3
        start = np.zeros(n3 + 1, np.uint32)
        tri = np.zeros(max(1, self.entries), np.uint32)
        check(native().dsim_mesh_grid(self.h, start, tri))
        return start, tri[:self.entries]

    def arrays(self):
        v = np.zeros(3 * self.nV, F)
        ti = np.zeros(3 * self.nT, np.uint32)
        check(native().dsim_mesh_arrays(self.h, v, ti))
        return v, ti

    def free(self):
        if self.h:
            native().dsim_mesh_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def mesh_params(stdDevs, T2, permeability, deltaTime, phaseConstant, reflectionType=1,
                spinRadius=0.005, maxSubsegments=0):
    p = _lib.MeshParams()
    p.stdDevs[:] = [float(x) for x in stdDevs]
    p.T2[:] = [float(x) for x in T2]
    p.permeability = float(permeability)
    p.reflectionType = int(reflectionType)
    p.spinRadius = float(spinRadius)
    p.deltaTime = float(deltaTime)
    p.phaseConstant = float(phaseConstant)
    p.maxSubsegments = int(maxSubsegments)
    return p


def mesh_run(mesh, spins, params, g=(0, 0, 0), iterations=1, seed=1, step0=0, draws=None,
             grad_per_step=None, count=False, scanned=False):
    gg = np.ascontiguousarray(g, F)
    d = None if draws is None else np.ascontiguousarray(draws, F).reshape(-1)
    gp = None if grad_per_step is None else np.ascontiguousarray(grad_per_step, F).reshape(-1)
    check(native().dsim_mesh_run(mesh.h, spins.h, C.byref(params), gg, gp, int(iterations),
                                 int(seed), int(step0), d, (1 if count else 0) | (2 if scanned else 0)))


class Cylinders:
    """Cylinder substrate (dSim2 fibers) with the reference's grid."""

    def __init__(self, handle):
        self.h = handle
        geom = np.zeros(3, np.uint32)
        L = C.c_float(0)
        check(native().dsim_cyl_info(self.h, geom, C.byref(L), None, None, None))
        self.numCubes, self.maxFPC, self.nF = [int(x) for x in geom]
        self.cubeLength = F(L.value)

    @classmethod
    def load(cls, path, spaceScale):
        h = C.c_void_p()
        check(native().dsim_cyl_load(str(path).encode(), float(spaceScale), C.byref(h)))
        return cls(h)

    @classmethod
    def from_arrays(cls, fiberPos4, maxRadius):
        fp = np.ascontiguousarray(fiberPos4, F).reshape(-1)
        h = C.c_void_p()
        check(native().dsim_cyl_create(fp, len(fp) // 4, float(maxRadius), C.byref(h)))
        return cls(h)

    def grid(self):
        geom = np.zeros(3, np.uint32)
        L = C.c_float(0)
        n3 = self.numCubes ** 3
        cc = np.zeros(n3, np.uint32)
        cubes = np.zeros(max(1, n3 * self.maxFPC), np.uint32)
        fp = np.zeros(max(1, 4 * self.nF), F)
        check(native().dsim_cyl_info(self.h, geom, C.byref(L), cc, cubes, fp))
        return cc, cubes, fp[:4 * self.nF]

    def set_fine(self, k):
        """Rebuild the fine filter grid with k cells per grid-cell edge (0: none)."""
        check(native().dsim_cyl_set_fine(self.h, int(k)))

    def fine_info(self):
        info = np.zeros(3, np.uint64)
        check(native().dsim_cyl_fine_info(self.h, info))
        return {"k": int(info[0]), "entries": int(info[1]), "nbytes": int(info[2])}

    def free(self):
        if self.h:
            native().dsim_cyl_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def cyl_params(intraAdc, extraAdc, myelinAdc, spaceScale, T2fiber, T2myelin, T2outside,
               permeability, innerRadiusProportion, deltaTime, phaseConstant, spinRadius=0.005):
    p = _lib.CylParams()
    p.intraAdc, p.extraAdc, p.myelinAdc = float(intraAdc), float(extraAdc), float(myelinAdc)
    p.spaceScale = float(spaceScale)
    p.T2fiber, p.T2myelin, p.T2outside = float(T2fiber), float(T2myelin), float(T2outside)
    p.permeability = float(permeability)
    p.innerRadiusProportion = float(innerRadiusProportion)
    p.spinRadius = float(spinRadius)
    p.deltaTime = float(deltaTime)
    p.phaseConstant = float(phaseConstant)
    return p


def cyl_run(cyl, spins, params, g=(0, 0, 0), iterations=1, seed=1, step0=0, draws=None,
            grad_per_step=None, count=False):
    gg = np.ascontiguousarray(g, F)
    d = None if draws is None else np.ascontiguousarray(draws, F).reshape(-1)
    gp = None if grad_per_step is None else np.ascontiguousarray(grad_per_step, F).reshape(-1)
    check(native().dsim_cyl_run(cyl.h, spins.h, C.byref(params), gg, gp, int(iterations),
                                int(seed), int(step0), d, 1 if count else 0))


WAVES = {"pgse": 0, "ogse": 1, "table": 2}


class Batch:
    """Many jobs advanced together (include/dsim_batch.h).  Each job keeps
    per-spin gradient moments; signal(job, gradScaled) evaluates any gradient
    that shares the job's waveform."""

    def __init__(self, spin_capacity, job_capacity=1024):
        self.h = C.c_void_p()
        check(native().dsim_batch_create(int(spin_capacity), int(job_capacity), C.byref(self.h)))
        self._keep = []

    def close(self):
        if self.h:
            native().dsim_batch_free(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_mesh(self, mesh):
        sid = C.c_uint32()
        check(native().dsim_batch_add_mesh(self.h, mesh.h, C.byref(sid)))
        self._keep.append(mesh)
        return sid.value

    def add_cyl(self, cyl):
        sid = C.c_uint32()
        check(native().dsim_batch_add_cyl(self.h, cyl.h, C.byref(sid)))
        self._keep.append(cyl)
        return sid.value

    def submit(self, substrate, pos, comp, fiber, steps, dt, step_sd, T2, phase_constant, seed,
               permeability=0.0, waveform="pgse", delta=0.0, Delta=0.0, frequency=0.0, table=None,
               reflection_type=1, spin_radius=0.005, inner_radius_proportion=1.0, precise=False, local=False):
        """precise: the FP64 step (DSIM_JOB_PRECISE); local: FP32 cell-local
        offsets with FP64 re-tests (DSIM_JOB_LOCAL)."""
        pos = np.ascontiguousarray(pos, F).reshape(-1)
        n = len(pos) // 3
        d, tab = _job_desc(substrate, n, steps, dt, step_sd, T2, phase_constant, seed, permeability, waveform,
                           delta, Delta, frequency, table, reflection_type, spin_radius,
                           inner_radius_proportion, precise, local)
        jid = C.c_uint32()
        comp = np.ascontiguousarray(comp, np.uint8)
        fib = None if fiber is None else np.ascontiguousarray(fiber, np.uint32)
        check(native().dsim_batch_submit(self.h, C.byref(d), pos, comp, fib, C.byref(jid)))
        return jid.value

    def configure(self, chunk=20, occupancy=4, graph_chunks=8, block=None):
        check(native().dsim_batch_configure(self.h, int(chunk), int(occupancy), int(graph_chunks)))
        if block is not None:
            check(native().dsim_batch_set_block(self.h, int(block)))

    def advance(self, steps):
        check(native().dsim_batch_advance(self.h, int(steps)))

    def run(self):
        check(native().dsim_batch_run(self.h))

    def sync(self):
        check(native().dsim_batch_sync(self.h))

    def job_status(self, job):
        s = C.c_uint32()
        d = C.c_int()
        check(native().dsim_batch_job_status(self.h, int(job), C.byref(s), C.byref(d)))
        return s.value, bool(d.value)

    def signal(self, job, grad_scaled, region=0.0):
        """FP64 sums (nG, 5, 3) of X, Y, n; region > 0 keeps spins inside
        +-region (dSim2 reads +-0.8)."""
        g = np.ascontiguousarray(grad_scaled, F).reshape(-1, 3)
        out = np.zeros(15 * len(g), np.float64)
        check(native().dsim_batch_signal_region(self.h, int(job), g.reshape(-1), len(g), float(region), out))
        return out.reshape(len(g), 5, 3)

    def get(self, job, n):
        pos = np.zeros(3 * n, F); mag = np.zeros(n, F); mom = np.zeros(6 * n, F)
        comp = np.zeros(n, np.uint8); fib = np.zeros(n, np.uint32)
        check(native().dsim_batch_get(self.h, int(job), pos, mag, mom, comp, fib))
        return pos, mag, mom.reshape(n, 6), comp, fib

    def counts(self, job):
        c = np.zeros(2, np.uint64)
        check(native().dsim_batch_counts(self.h, int(job), c))
        return c

    def status(self):
        return int(native().dsim_batch_status(self.h))

    def precision_counts(self, job):
        """{fine-grid records examined, FP64 triangle tests} of a precision-form job."""
        c = np.zeros(2, np.uint64)
        check(native().dsim_batch_precision_counts(self.h, int(job), c))
        return int(c[0]), int(c[1])

    def get_precise(self, job, n):
        """FP64 positions (n x 3) and magnitudes of a precision-form or
        cell-local job, in spin order."""
        pos = np.zeros(3 * n, np.float64); mag = np.zeros(n, np.float64)
        check(native().dsim_batch_get_precise(self.h, int(job), pos, mag))
        return pos.reshape(n, 3), mag

    def retire(self, job):
        check(native().dsim_batch_retire(self.h, int(job)))

    def compact(self):
        check(native().dsim_batch_compact(self.h))

    def autotune(self, trial_steps=40):
        """Times every candidate configuration on a snapshot; returns
        ({occupancy, chunk, fine_cells_per_ref_cell, block}, ms)."""
        best = np.zeros(3, np.uint32)
        ms = C.c_float()
        check(native().dsim_batch_autotune(self.h, int(trial_steps), best, C.byref(ms)))
        th = C.c_uint32()
        check(native().dsim_batch_block(self.h, C.byref(th)))
        return {"occupancy": int(best[0]), "chunk": int(best[1]), "fine_per_ref": best[2] / 2.0,
                "block": int(th.value)}, ms.value

    def info(self):
        a = np.zeros(6, np.uint64)
        check(native().dsim_batch_info(self.h, a))
        keys = ("spins", "jobs", "running", "bytes", "launches", "graph_launches")
        return dict(zip(keys, [int(x) for x in a]))


def pgse_table(steps, dt, delta, Delta):
    """The DSIM_WAVE_PGSE waveform as a table: +1 on [0, nd), -1 on [nD, nD + nd)."""
    w = np.zeros(steps, F)
    nd, nD = int(round(delta / dt)), int(round(Delta / dt))
    w[:min(nd, steps)] = 1
    w[nD:min(nD + nd, steps)] = -1
    return w


def _job_desc(substrate, n, steps, dt, step_sd, T2, phase_constant, seed, permeability=0.0,
              waveform="pgse", delta=0.0, Delta=0.0, frequency=0.0, table=None, reflection_type=1,
              spin_radius=0.005, inner_radius_proportion=1.0, precise=False, local=False):
    d = _lib.JobDesc()
    d.substrate, d.nSpins, d.steps = int(substrate), int(n), int(steps)
    d.deltaTime = float(dt)
    sd = list(np.asarray(step_sd, F).reshape(-1)) + [0.0] * 4
    t2 = list(np.asarray(T2, F).reshape(-1)) + [0.0] * 4
    d.stepSd[:] = [float(x) for x in sd[:4]]
    d.T2[:] = [float(x) for x in t2[:4]]
    d.permeability = float(permeability)
    d.reflectionType = int(reflection_type)
    d.spinRadius = float(spin_radius)
    d.innerRadiusProportion = float(inner_radius_proportion)
    d.phaseConstant = float(phase_constant)
    d.waveform = WAVES[waveform]
    d.delta, d.Delta, d.frequency = float(delta), float(Delta), float(frequency)
    tab = None
    if table is not None:
        tab = np.ascontiguousarray(table, F)
        assert len(tab) >= steps
        d.table = tab.ctypes.data
    d.seed = int(seed)
    d.flags = (1 if precise else 0) | (2 if local else 0)
    return d, tab


class Server:
    """Continuous-batching request loop (include/dsim_serve.h)."""

    def __init__(self, spin_capacity, job_capacity=1024, hbm_cap=150e9):
        self.h = C.c_void_p()
        check(native().dsim_server_create(int(spin_capacity), int(job_capacity), int(hbm_cap), C.byref(self.h)))
        self._keep = []
        self.nG = {}

    def add_mesh(self, mesh):
        sid = C.c_uint32()
        check(native().dsim_server_add_mesh(self.h, mesh.h, C.byref(sid)))
        self._keep.append(mesh)
        return sid.value

    def add_cyl(self, cyl):
        sid = C.c_uint32()
        check(native().dsim_server_add_cyl(self.h, cyl.h, C.byref(sid)))
        self._keep.append(cyl)
        return sid.value

    def configure(self, chunk=20, occupancy=4, graph_chunks=8):
        check(native().dsim_server_configure(self.h, int(chunk), int(occupancy), int(graph_chunks)))

    def start(self):
        check(native().dsim_server_start(self.h))

    def submit(self, substrate, pos, comp, fiber, grad_scaled, steps, dt, step_sd, T2, phase_constant, seed,
               **kw):
        pos = np.ascontiguousarray(pos, F).reshape(-1)
        n = len(pos) // 3
        d, tab = _job_desc(substrate, n, steps, dt, step_sd, T2, phase_constant, seed, **kw)
        g = np.ascontiguousarray(grad_scaled, F).reshape(-1)
        comp = np.ascontiguousarray(comp, np.uint8)
        fib = None if fiber is None else np.ascontiguousarray(fiber, np.uint32)
        t = C.c_uint32()
        check(native().dsim_server_submit(self.h, C.byref(d), pos, comp, fib, g, len(g) // 3, C.byref(t)))
        self.nG[t.value] = len(g) // 3
        return t.value

    def poll(self, ticket):
        """(done, signals (nG, 5, 3) or None, times {submit, admit, done})"""
        done = C.c_int()
        out = np.zeros(15 * self.nG[ticket], np.float64)
        times = np.zeros(3, np.float64)
        check(native().dsim_server_poll(self.h, int(ticket), C.byref(done), out, times))
        return bool(done.value), (out.reshape(-1, 5, 3) if done.value else None), times

    def drain(self):
        check(native().dsim_server_drain(self.h))

    def stop(self):
        check(native().dsim_server_stop(self.h))

    def stats(self):
        a = np.zeros(8, np.float64)
        check(native().dsim_server_stats(self.h, a))
        keys = ("jobs_done", "spin_steps", "busy_s", "max_inflight", "hbm_peak", "quanta", "compactions",
                "errors")
        return dict(zip(keys, a.tolist()))

    def close(self):
        if self.h:
            native().dsim_server_free(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def rng_draws(seed, spin0, step, n, stream=0):
    """The step kernels' draws (n.x, n.y, n.z, u) for spins [spin0, spin0 + n)
    at global step `step` (Philox key = seed, counter word 3 = stream)."""
    out = np.zeros(4 * n, F)
    check(native().dsim_rng_draws(int(seed), int(spin0), int(step), int(stream), int(n), None, out))
    return out.reshape(n, 4)


# ---- the simulate call: config, gradients, sequencer, tensor fit ------------
def load_config(path):
    """sim.cfg (dSim3 or dSim2 keys) as a dict."""
    c = _lib.Config()
    check(native().dsim_config_load(str(path).encode(), C.byref(c)))
    out = {}
    for name, _ in c._fields_:
        v = getattr(c, name)
        out[name] = v.decode() if isinstance(v, bytes) else v
    return out


def parse_grads(path=None, text=None):
    """Gradient rows [n, 6]: delta, Delta, readout (ms), Gx, Gy, Gz (mT/m)."""
    n = C.c_uint32()
    if path is not None:
        f = native().dsim_grads_parse_file
        arg = str(path).encode()
    else:
        f = native().dsim_grads_parse_string
        arg = str(text).encode()
    check(f(arg, None, 0, C.byref(n)))
    rows = np.zeros(6 * max(n.value, 1), F)
    check(f(arg, rows, n.value, C.byref(n)))
    return rows[:6 * n.value].reshape(-1, 6)


def pgse_schedule(row, dt, steps_per_update):
    """Per-step gradient (mT/m) of one sequencer run, [steps, 3]."""
    r = np.ascontiguousarray(row, F)
    n = C.c_uint32()
    check(native().dsim_pgse_schedule(r, float(dt), int(steps_per_update), None, 0, C.byref(n)))
    g = np.zeros(3 * max(n.value, 1), F)
    check(native().dsim_pgse_schedule(r, float(dt), int(steps_per_update), g, n.value, C.byref(n)))
    return g[:3 * n.value].reshape(-1, 3)


def tensor_fit(rows, signal):
    """{tensor, eigvecs (columns), eigvals ascending, md, fa, rd}."""
    rows = np.ascontiguousarray(rows, F).reshape(-1)
    sig = np.ascontiguousarray(signal, np.float64)
    T = np.zeros(9); E = np.zeros(9); ev = np.zeros(3, F)
    md, fa, rd = C.c_float(), C.c_float(), C.c_float()
    check(native().dsim_tensor_fit(rows, sig, len(sig), T, E, ev, C.byref(md), C.byref(fa), C.byref(rd)))
    return {"tensor": T.reshape(3, 3), "eigvecs": E.reshape(3, 3), "eigvals": ev, "md": md.value, "fa": fa.value,
            "rd": rd.value}


def write_results(out_path, config, rows, signals, seconds=0.0):
    """Append the reference's results block (dsim_write_results) for gradient
    rows [n, 6] and signals [n, 5]; config: a dict as load_config returns."""
    c = _lib.Config()
    for name, _ in c._fields_:
        if name in config:
            v = config[name]
            setattr(c, name, v.encode() if isinstance(v, str) else v)
    r = np.ascontiguousarray(rows, F).reshape(-1)
    sg = np.ascontiguousarray(signals, np.float64).reshape(-1)
    check(native().dsim_write_results(str(out_path).encode(), C.byref(c), r, sg, len(r) // 6, float(seconds)))


def simulate(cfg_path, seed=1, shared_walk=False, write_out=False, cap=4096):
    """Run a sim.cfg on the GPU: (signals [nG, 5], seconds)."""
    out = np.zeros(5 * cap, np.float64)
    n = C.c_uint32()
    sec = C.c_double()
    flags = (1 if shared_walk else 0) | (2 if write_out else 0)
    check(native().dsim_simulate(str(cfg_path).encode(), int(seed), flags, out, cap, C.byref(n), C.byref(sec)))
    return out[:5 * n.value].reshape(-1, 5), sec.value
