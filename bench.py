#!/usr/bin/env python3
"""Throughput of the mesh hot path on one GB300 (spin-steps/s).

Workload (the reference's mesh-scale plain configuration): 400 beaded axons
tessellated with 32 vertices per ring and a ring every 0.5 um over 50 um
(2.56M triangles), base radius LogNormal(median 1 um, sigma 0.4) clipped to
[0.5, 3] um, 20 % sinusoidal beading with a 10 um period, reflecting glia
membranes, in a 50 um cube (spaceScale 25, 50^3 grid of 1 um cells);
1,048,576 spins; D = 2.0 um^2/ms; dt = 5 us; PGSE delta 15 ms, Delta 40 ms,
b = 3000 s/mm^2 along one Fibonacci direction.  Synthetic substrate and
spins, seeded.  One bench step = one launch advancing every spin 1000 time
steps (1.05e9 spin-steps); K steps cover the 10,000-step unit of work.

Reported: value = spin-steps/s from CUDA events around each launch on the
engine's stream (L2 flushed between launches); e2e = the same through the
reference-facing dSim3 C-ABI (libdsim3.so), with the reference host loop's
copies (state to the device, integrateSystem, state back) from pinned host
buffers inside the timed region; roofline of the step kernel; CPU baseline
of the oracle port on a bounded sample.

--impl reference times the reference's CPU algorithm (the oracle port of
dSim3's cpuIntegrate, all host threads) on a bounded sample of the same
workload; the oracle also builds that arm's mesh arrays and grid (initFibers
and populateCubes from a mesh file of the workload), so it makes no GPU call.  Multi-GPU (--gpus N under torchrun): independent replicas, one
per rank, no collective on the data path (weak scaling).
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

F = np.float32
DRAM_BYTES_PER_SPIN_STEP = 2.9018e9 / (262144 * 60)
METRIC = "spin-steps/s on 1 GB300, served vs plain, at \u22641e-3 signal err; p50/p99 latency"
UNIT = "spin-steps/s"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# --------------------------------------------------------------------------
# workload
# --------------------------------------------------------------------------
class Workload:
    def __init__(self, axons=400, spins=1 << 20, seed=1):
        from dsim_gb300 import substrates as S
        from dsim_gb300.engine import grad_scaled, phase_constant, std_devs
        t0 = time.time()
        self.axons = axons
        self.tube = S.beaded_tubes(n_axons=axons, verts_per_ring=32, ring_spacing=0.5, length=50.0,
                                   box=50.0, seed=seed, membranes="G", allow_overlap=True)
        self.spaceScale = 25.0
        self.numCubes = 50
        self.N = spins
        self.D, self.dt = 2.0, 0.005
        self.delta, self.Delta = 15.0, 40.0
        self.steps_per_launch = 1000
        rng = np.random.default_rng(seed + 1)
        pos = rng.uniform(-0.99, 0.99, (self.N, 3)).astype(F)
        self.pos = pos.reshape(-1).copy()
        self.comp, self.fiber = self._compartments(pos)
        self.stdDevs = std_devs(self.D, self.D, 0.1 * self.D, self.spaceScale, self.dt)
        self.T2 = np.array([80.0, 80.0, 7.5, 80.0], F)
        self.pc = phase_constant(42576.0, self.dt)
        # b = 3000 s/mm^2 = 3 ms/um^2, first direction of a 64-point Fibonacci sphere
        b = 3.0
        gmag = np.sqrt(b / (self.Delta - self.delta / 3.0)) / (2 * np.pi * 42576.0 * 1e-9 * self.delta)
        k = 0.5
        zc = 1 - 2 * k / 64
        rr = np.sqrt(1 - zc * zc)
        phi = np.pi * (3 - np.sqrt(5)) * k
        self.G = gmag * np.array([rr * np.cos(phi), rr * np.sin(phi), zc])
        self.g = grad_scaled(self.G, self.spaceScale)
        nd, nD = int(round(self.delta / self.dt)), int(round(self.Delta / self.dt))
        self.total_steps = 10000
        w = np.zeros(self.total_steps, F)
        w[:nd] = 1
        w[nD:nD + nd] = -1
        self.wave = w
        self.grad = (w[:, None] * self.g[None, :]).astype(F)
        log("workload: %d triangles, %d vertices, overlap=%s, %.1fs" % (
            len(self.tube["trgls"]), len(self.tube["vertices"]), self.tube["overlap"], time.time() - t0))

    def _compartments(self, pos):
        um = pos.astype(np.float64) * self.spaceScale
        comp = np.zeros(len(pos), np.uint8)
        fib = np.full(len(pos), 0xFFFF, np.uint16)
        cx, cy = self.tube["centres"][:, 0], self.tube["centres"][:, 1]
        r0 = self.tube["radii"]
        # cells of 2 um to find candidate tubes
        for i in range(len(r0)):
            rz = r0[i] * (1 + 0.2 * np.sin(2 * np.pi * um[:, 2] / 10.0))
            sel = (np.abs(um[:, 0] - cx[i]) < rz) & (np.abs(um[:, 1] - cy[i]) < rz)
            sel &= np.hypot(um[:, 0] - cx[i], um[:, 1] - cy[i]) < rz * np.cos(np.pi / 32)
            sel &= comp == 0
            comp[sel] = 3
            fib[sel] = i
        return comp, fib


def make_mesh(W):
    from dsim_gb300.engine import Mesh
    t0 = time.time()
    m = Mesh.from_arrays(W.tube["vertices"], W.tube["trgls"], W.tube["membrane"], W.tube["fiber"],
                         W.spaceScale, W.numCubes)
    log("mesh on device: %d entries, max %d per cell, %.1f MB, built in %.2fs" % (
        m.entries, m.max_per_cell, m.nbytes / 1e6, time.time() - t0))
    return m


def mesh_params_of(W):
    from dsim_gb300.engine import mesh_params
    return mesh_params(W.stdDevs, W.T2, 0.0, W.dt, W.pc)


# --------------------------------------------------------------------------
# clocks during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm = [float(s[1]) for s in self.samples if len(s) > 2 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) > 2 and s[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            for k, n in enumerate(names):
                if len(s) > 5 + k and s[5 + k] == "Active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# --------------------------------------------------------------------------
# CPU baseline: the oracle port of dSim3's cpuIntegrate on a bounded sample
# --------------------------------------------------------------------------
def device_arrays(W, m):
    """The reference's mesh arrays for the oracle, from the device mesh: its
    vertices and grid (pinned equal to initFibers / populateCubes), helpers
    recomputed in the reference's expression order."""
    start, tri = m.grid()
    counts = np.diff(start.astype(np.int64)).astype(np.uint32)
    maxtpc = int(counts.max())
    dense = np.zeros((len(counts), maxtpc), np.uint32)
    idx = np.repeat(np.arange(len(counts)), counts)
    off = np.arange(len(tri)) - np.repeat(start[:-1].astype(np.int64), counts)
    dense[idx, off] = tri
    v, ti = m.arrays()
    H = _helpers(v, W.tube["trgls"].reshape(-1))
    return v, H, ti, counts, dense.reshape(-1), maxtpc, "mesh, grid and draws as on the GPU"


def oracle_arrays(W):
    """The reference's mesh arrays built on the host by the oracle alone: the
    workload written as a dSim3 mesh file and read back by the restatement of
    initFibers, the grid by the restatement of populateCubes."""
    import tempfile
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from dsim_gb300 import substrates as S
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "workload.mesh")
        S.write_mesh_file(path, W.tube)
        mo = O.Mesh(path, W.spaceScale)
    cc, tic, maxtpc = O.populate_cubes(mo.vertices, mo.trgls, W.numCubes)
    return (mo.vertices, mo.helpers, mo.triInfo, cc, tic, maxtpc,
            "mesh read and grid built by the oracle's initFibers / populateCubes")


def cpu_sample(W, arrays, threads, budget_s=12.0):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    v, H, ti, counts, dense, maxtpc, source = arrays
    p = O.params3(W.stdDevs, W.T2, 0.0, W.dt, W.numCubes, maxtpc)
    n = min(W.N, 4096 if threads == 1 else 4096 * threads)
    sel = np.random.default_rng(5).choice(W.N, n, replace=False)
    pos = W.pos.reshape(-1, 3)[sel].reshape(-1).copy()
    seed = np.random.default_rng(6).integers(1, 2 ** 32 - 1, 2 * n, dtype=np.uint64).astype(np.uint32)
    mag = np.ones(n, F)
    ph = np.zeros(n, F)
    comp = W.comp[sel].copy()
    fib = W.fiber[sel].copy()
    L = O.lib()
    # calibrate, then run ~budget seconds
    t0 = time.perf_counter()
    L.or3_integrate_mt(p, n, pos, seed, mag, ph, comp, fib, v, H, ti, counts, dense,
                       float(W.g[0]), float(W.g[1]), float(W.g[2]), float(W.pc), 5, threads)
    dt5 = time.perf_counter() - t0
    iters = max(5, int(budget_s / max(dt5 / 5, 1e-6)))
    t0 = time.perf_counter()
    L.or3_integrate_mt(p, n, pos, seed, mag, ph, comp, fib, v, H, ti, counts, dense,
                       float(W.g[0]), float(W.g[1]), float(W.g[2]), float(W.pc), iters, threads)
    el = time.perf_counter() - t0
    rate = n * iters / el
    return rate, "%d spins x %d steps of the workload (%s; %.1f s)" % (n, iters, source, el)


def _helpers(v, trgls):
    """Triangle helpers in float32 with the reference's expression order
    (dSim3/src/spinSystem.cpp:612-648)."""
    V = v.reshape(-1, 3)
    T = trgls.reshape(-1, 3)
    p1, p2, p3 = V[T[:, 0]], V[T[:, 1]], V[T[:, 2]]
    x1, y1, z1 = p1[:, 0], p1[:, 1], p1[:, 2]
    x2, y2, z2 = p2[:, 0], p2[:, 1], p2[:, 2]
    x3, y3, z3 = p3[:, 0], p3[:, 1], p3[:, 2]
    nx = (y2 - y1) * (z3 - z1) - (z2 - z1) * (y3 - y1)
    ny = (z2 - z1) * (x3 - x1) - (x2 - x1) * (z3 - z1)
    nz = (x2 - x1) * (y3 - y1) - (y2 - y1) * (x3 - x1)
    ln = np.sqrt(nx * nx + ny * ny + nz * nz)
    H = np.stack([nx / ln, ny / ln, nz / ln, x3 - x1, y3 - y1, z3 - z1, x2 - x1, y2 - y1, z2 - z1,
                  (x3 - x1) * (x2 - x1) + (y3 - y1) * (y2 - y1) + (z3 - z1) * (z2 - z1),
                  (x3 - x1) * (x3 - x1) + (y3 - y1) * (y3 - y1) + (z3 - z1) * (z3 - z1),
                  (x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1) + (z2 - z1) * (z2 - z1)], -1)
    return np.ascontiguousarray(H.astype(F).reshape(-1))


# --------------------------------------------------------------------------
# e2e through the reference-facing dSim3 C-ABI
# --------------------------------------------------------------------------
def e2e_abi3(W, m, steps, warmup, pinned):
    """The headline walk through the reference-facing dSim3 C-ABI
    (libdsim3.so), as a host that keeps the spin state in its own memory
    drives it: every call copies pos, randSeed and spinData from pinned host
    buffers to the device, runs integrateSystem for one 1000-step update with
    that update's PGSE gradient, and copies all three back (so each spin's
    Philox key, advanced by the call, goes into the next call).  The timed
    calls start from the same reset as the device-timed leg and walk the same
    steps; L2 is flushed before each call, outside its timed interval."""
    import ctypes as C
    from dsim_gb300 import _lib
    from dsim_gb300.engine import Spins
    L = _lib.abi3()
    start, tri = m.grid()
    counts = np.diff(start.astype(np.int64)).astype(np.uint32)
    maxtpc = int(counts.max())
    dense = np.zeros((len(counts), maxtpc), np.uint32)
    idx = np.repeat(np.arange(len(counts)), counts)
    off = np.arange(len(tri)) - np.repeat(start[:-1].astype(np.int64), counts)
    dense[idx, off] = tri
    v, ti = m.arrays()
    H = _helpers(v, W.tube["trgls"].reshape(-1))

    allocs = []

    def dev(arr):
        p = C.c_void_p()
        L.allocateArray(C.byref(p), arr.nbytes)
        L.copyArrayToDevice(p, arr.ctypes.data, 0, arr.nbytes)
        allocs.append(p)
        return p

    dV, dH, dTI = dev(v), dev(H), dev(ti)
    L.bindVertices(dV, len(v)); L.bindTriangleHelpers(dH, len(H)); L.bindTriInfo(dTI, len(ti))
    dTic, dCc = dev(dense.reshape(-1)), dev(counts)
    for name, val, ty in (("k_numCubes", W.numCubes, np.uint32), ("k_totalNumCubes", W.numCubes ** 3, np.uint32),
                          ("k_maxTrianglesPerCube", maxtpc, np.uint32),
                          ("k_cubeLength", F(2.0) / F(W.numCubes), F), ("k_reflectionType", 1, np.uint32),
                          ("k_permeability", 0.0, F), ("k_deltaTime", W.dt, F)):
        a = np.array([val], ty)
        L.copyConstantToDevice(name.encode(), a.ctypes.data, 0, 4)
    for name, tab in (("k_T2Values", W.T2), ("k_stdDevs", W.stdDevs)):
        a = np.ascontiguousarray(tab, F)
        L.copyConstantToDevice(name.encode(), a.ctypes.data, 0, 16)
    N = W.N
    spins = np.zeros(N, np.dtype([("mag", "<f4"), ("phase", "<f4"), ("comp", "u1"), ("pad", "u1"),
                                  ("fiber", "<u2")]))
    spins["mag"] = 1.0
    spins["comp"], spins["fiber"] = W.comp, W.fiber
    seeds = np.random.default_rng(9).integers(1, 2 ** 32 - 1, 2 * N, dtype=np.uint64).astype(np.uint32)
    hpos, hseed, hspin = pinned(W.pos.nbytes), pinned(seeds.nbytes), pinned(spins.nbytes)
    dPos, dSeed, dSpin = dev(W.pos), dev(seeds), dev(spins)
    flusher = Spins(1)
    it = W.steps_per_launch

    def reset():
        hpos[:] = W.pos.view(np.uint8)
        hseed[:] = seeds.view(np.uint8)
        hspin[:] = spins.view(np.uint8)

    def one(k):
        # the update's gradient: the PGSE waveform is constant over each 1000-step update
        lo = (k * it) % W.total_steps
        assert np.all(W.wave[lo:lo + it] == W.wave[lo])
        g = _lib.Float3(*[float(F(W.wave[lo] * x)) for x in W.g])
        L.copyArrayToDevice(dPos, hpos.ctypes.data, 0, hpos.nbytes)
        L.copyArrayToDevice(dSeed, hseed.ctypes.data, 0, hseed.nbytes)
        L.copyArrayToDevice(dSpin, hspin.ctypes.data, 0, hspin.nbytes)
        L.integrateSystem(dPos, dSeed, dSpin, float(W.dt), 0.0, N, g, float(W.pc), it, dTic, dCc)
        L.copyArrayFromDevice(hpos.ctypes.data, dPos, 0, hpos.nbytes)
        L.copyArrayFromDevice(hseed.ctypes.data, dSeed, 0, hseed.nbytes)
        L.copyArrayFromDevice(hspin.ctypes.data, dSpin, 0, hspin.nbytes)

    reset()
    for k in range(warmup):
        one(k)
    L.threadSync()
    reset()
    per = []
    for k in range(steps):
        flusher.flush_l2(512 << 20)
        flusher.sync()
        L.threadSync()
        t0 = time.perf_counter()
        one(k)
        L.threadSync()
        per.append(time.perf_counter() - t0)
    el = sum(per)
    st = L.dsim3_last_status()
    if st != 0:
        raise RuntimeError("dSim3 ABI: %s" % L.dsim3_last_error())
    out = np.frombuffer(hspin.tobytes(), spins.dtype)
    X = (out["mag"].astype(np.float64) * np.cos(out["phase"].astype(np.float64))).sum()
    Y = (out["mag"].astype(np.float64) * np.sin(out["phase"].astype(np.float64))).sum()
    for p in allocs:
        L.freeArray(p)
    flusher.free()
    return {"value": steps * it * N / el, "unit": UNIT, "h2d_bytes_per_step": int(hpos.nbytes + hseed.nbytes + hspin.nbytes),
            "d2h_bytes_per_step": int(hpos.nbytes + hseed.nbytes + hspin.nbytes), "ms_per_step": 1e3 * el / steps,
            "calls": steps, "steps_walked": [0, steps * it], "l2": "flushed before each call (untimed)",
            "signal_after_run": float(np.hypot(X, Y) / N),
            "path": "libdsim3.so integrateSystem; pos, randSeed, spinData copied in and out of pinned host buffers "
                    "every call"}


def pinned_factory():
    try:
        import torch
        if torch.cuda.is_available():
            def pinned(nbytes):
                return torch.empty(nbytes, dtype=torch.uint8, pin_memory=True).numpy()
            return pinned, True
    except Exception:
        pass
    return (lambda nbytes: np.empty(nbytes, np.uint8)), False


# --------------------------------------------------------------------------
def run_mix_only(args):
    """--mix-only FORM: the 48-job mix of the forms leg in one batch, once, in
    FORM ("fp32" or "bar"), configured by --mix-config (else autotuned); for
    profiling the batch step kernels on their own."""
    W = Workload(axons=args.axons, spins=4096, seed=1)
    m = make_mesh(W)
    subs, mix = build_mix(W, m, args.mix_jobs, 11, (4096, args.mix_max_spins),
                          (args.mix_min_steps, args.mix_max_steps))
    if args.mix_config:
        cfg = {"occupancy": args.mix_config[0], "chunk": args.mix_config[1], "block": args.mix_block}
    else:
        best, _ = tune_mix(subs, mix)
        cfg = {"occupancy": best["occupancy"], "chunk": best["chunk"], "block": best.get("block")}
    work = sum(j["n"] * j["steps"] for j in mix)
    el, sigs, info, st = run_batched_mix(subs, mix, cfg, form=args.mix_only)
    return {"metric": "spin-steps/s", "value": work / el, "unit": "spin-steps/s", "form": args.mix_only,
            "config": dict(cfg, jobs=len(mix), spin_steps=work), "seconds": el, "kernel_launches": info["launches"],
            "status": st}


def run_ours(args, rank, world):
    from dsim_gb300.engine import DeviceInfo, Spins, mesh_run
    dev = DeviceInfo()
    W = Workload(axons=args.axons, spins=args.spins, seed=1 + rank)
    W.steps_per_launch = args.steps_per_launch
    m = make_mesh(W)
    if args.kernel > 0:
        m.set_kernel(args.kernel)
    if args.records > 0:
        m.set_records(args.records)
    if args.accel >= 0:
        m.set_accel(args.accel)
    acc_info = m.accel_info()
    log("accel grid: %s" % acc_info)
    p = mesh_params_of(W)
    s = Spins(W.N)
    if args.sort_every >= 0:
        s.set_sort_interval(args.sort_every)
    it = W.steps_per_launch

    def reset():
        s.set(W.pos, np.ones(W.N, F), np.zeros(W.N, F), W.comp, W.fiber)

    # T-bar and per-step statistics on an untimed launch with counters on
    reset()
    mesh_run(m, s, p, grad_per_step=W.grad[:it], iterations=it, seed=11, step0=0, count=True, scanned=True)
    scanned = s.scanned(reset=True).astype(np.float64)
    cnt = s.counts(reset=True)
    Tbar = scanned.sum() / (W.N * it)
    refl_per_step = cnt[:, 0].sum() / (W.N * it)
    if s.status() != 0:
        raise RuntimeError("kernel status flags set")
    # warm-up
    reset()
    for k in range(args.warmup):
        mesh_run(m, s, p, grad_per_step=W.grad[(k * it) % W.total_steps:][:it], iterations=it, seed=3,
                 step0=k * it)
    s.sync()
    reset()
    s.launches(reset=True)
    times = []
    barrier(world)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", 0))) as clk:
        for k in range(args.steps):
            s.flush_l2(512 << 20)
            s.timer_start()
            lo = (k * it) % W.total_steps
            mesh_run(m, s, p, grad_per_step=W.grad[lo:lo + it], iterations=it, seed=1, step0=k * it)
            times.append(s.timer_stop())
        s.sync()
    barrier(world)
    launches = s.launches(reset=True)
    assert s.status() == 0
    total_ms = sum(times)
    total_ms = max_over_ranks(total_ms, world)
    spin_steps = args.steps * it * W.N * world
    value = spin_steps / (total_ms / 1e3)
    # signal after the unit of work (sanity, reported)
    sums = s.signal()
    from dsim_gb300.engine import signal_from_sums
    S = signal_from_sums(sums)[0]

    hbm, kind = peaks()
    # DRAM bytes of the step kernel per spin-step, from one ncu capture of
    # k_mesh_step_flat<0,6,1,1,0> (kernel 8 at 6 blocks per SM, 112^3 fine grid, 32-byte
    # records) on 262,144 spins x 60 steps of this mesh: 2.7997 GB read + 0.1021 GB
    # written per launch = 184.5 B per spin-step; scaled to this call's spin-steps
    default_cfg = args.kernel <= 0 and args.accel < 0 and args.records <= 0 and args.sort_every < 0
    traffic = DRAM_BYTES_PER_SPIN_STEP * it * W.N if default_cfg else None
    traffic_note = ("bytes per launch (one %d-step call) = 184.5 B per spin-step from an ncu capture of "
                    "the default step kernel (at 6 blocks per SM), scaled by spin-steps" % it) if default_cfg else "no capture for this configuration"
    S_bytes = 12 + 4 + 4
    B_step = 2 * S_bytes + 40 * Tbar
    mean_launch_ms = (sum(times) / len(times))
    achieved = B_step * (it * W.N) / (mean_launch_ms / 1e3) / 1e9
    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "mesh: %d beaded tubes, %d triangles, 50 um cube, 1 um cells, %d spins, "
                               "dt 5 us, PGSE delta 15 Delta 40 ms, b 3000 s/mm2, %d steps per launch"
                               % (W.axons, len(W.tube["trgls"]), W.N, it),
                   "spins": W.N, "triangles": int(len(W.tube["trgls"])), "steps_per_launch": it,
                   "form": "plain", "rng": "philox4x32-10", "l2": "flushed between launches (512 MB write)",
                   "parallelism": "replicas" if world > 1 else "single",
                   "accel_cells_per_axis": acc_info["cells"], "sort_every": args.sort_every},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic, "peak_kind": kind,
                     "traffic_note": traffic_note,
                     "bytes_per_spin_step": B_step, "T_bar": Tbar,
                     "note": "B_step = 2*S + 40*T_bar, S = 20 B, T_bar = grid entries scanned per step (kernel counter)"},
        "gpu_launches": launches,
        "launch_ms": times,
        "clocks": clk.summary(),
        "device": dev.name,
        "signal_after_run": S,
        "reflections_per_step": refl_per_step,
    }
    if rank == 0 and not args.no_e2e:
        pinned, is_pinned = pinned_factory()
        e = e2e_abi3(W, m, args.steps, args.warmup, pinned)
        e["pinned"] = is_pinned
        res["e2e"] = e
    if rank == 0 and not args.no_err:
        res["err_vs_fp64"] = run_headline_error(args, W, m)
    if rank == 0 and not args.no_forms:
        res["forms"] = run_forms(args, W, m)
    if rank == 0 and not args.no_precision:
        res["precision"] = run_precision(args, W, m)
    # the precision configuration at full size runs by default on one GPU
    # (about two minutes: 1M spins x 20,000 steps x 3 waveforms in each form)
    if rank == 0 and (args.c5_full or (world == 1 and not args.no_c5_full)):
        res["precision_full"] = run_precision_full(args, W, m)
    if rank == 0 and args.c4_full:
        res["serving_full"] = run_c4_full(args, W, m)
    if rank == 0 and not args.no_cylinders:
        res["cylinders"] = run_cylinders(args)
    if rank == 0 and not args.no_cpu:
        threads = 1
        rate, sample = cpu_sample(W, device_arrays(W, m), threads, budget_s=args.cpu_seconds)
        res["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": sample}
    return res


def run_reference(args, rank, world):
    if rank != 0:
        return None
    # host cores only: the oracle builds the mesh arrays and the grid, no GPU call
    W = Workload(axons=args.axons, spins=args.spins, seed=1)
    threads = os.cpu_count() or 1
    rate, sample = cpu_sample(W, oracle_arrays(W), threads, budget_s=args.cpu_seconds)
    return {"impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "mesh: %d beaded tubes, %d triangles, %d spins (sampled)" % (
                W.axons, len(W.tube["trgls"]), W.N)},
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# --------------------------------------------------------------------------
# signal error against an FP64 run on the same draws
# --------------------------------------------------------------------------
ERR_BAR = 1e-3


def _z_from_moments(mag, mom6, gs, pc):
    """Per-spin m e^{i phi} for every gradient from a batch job's moments
    (phi = pc g . M, M = moment - its Kahan compensation)."""
    M = mom6[:, :3].astype(np.float64) - mom6[:, 3:].astype(np.float64)
    return mag.astype(np.float64)[:, None] * np.exp(1j * float(pc) * (M @ np.asarray(gs, np.float64).reshape(-1, 3).T))


def _S(z, sel=None):
    if sel is not None:
        z = z[sel]
    return np.abs(z.sum(0)) / max(len(z), 1)


def _err_summary(dS, what):
    dS = np.asarray(dS, np.float64).reshape(-1)
    return {"max_abs_dS": float(dS.max()), "median_abs_dS": float(np.median(dS)), "gradients": int(len(dS)),
            "within_1e-3": bool(dS.max() <= ERR_BAR), "against": what}


def philox_draw_chunks(seed, n, steps, chunk=500):
    """The step kernels' own draws for spins [0, n) of a job keyed by `seed`,
    [steps][n][4], yielded `chunk` steps at a time."""
    from dsim_gb300.engine import rng_draws
    for t0 in range(0, steps, chunk):
        t1 = min(steps, t0 + chunk)
        yield t0, np.stack([rng_draws(seed, 0, t, n) for t in range(t0, t1)])


def cyl_fp64_z(cyl, pos3, imo, near, step_sd_adc, T2, perm, inner, dt, pc, grads, wave, seed):
    """FP64 oracle walk (restated dSim2 step in double, oracle/) of a
    cylinder job's spins on the GPU's Philox draws for that job: per-spin
    m e^{i phi} [n][nG] and final positions."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    cc, cubes, fp = cyl.grid()
    P = O.Params2()
    P.intraAdcScaled, P.myelinAdcScaled, P.extraAdcScaled = [F(a) for a in step_sd_adc]
    P.T2fiber, P.T2myelin, P.T2outside = [float(x) if x > 0 else 1e30 for x in T2[:3]]
    P.permeability, P.innerRadiusProportion, P.spinRadius, P.deltaTime = float(perm), float(inner), 0.005, float(dt)
    P.numCubes, P.maxFibersPerCube, P.cubeLength = cyl.numCubes, cyl.maxFPC, cyl.cubeLength
    n = len(imo)
    pos = np.ascontiguousarray(pos3, np.float64).reshape(-1).copy()
    mag = np.ones(n, np.float64)
    im = np.ascontiguousarray(imo, np.uint32).copy()
    nr = np.ascontiguousarray(near, np.uint32).copy()
    ph = np.zeros((n, len(np.asarray(grads).reshape(-1, 3))), np.float64)
    for t0, d in philox_draw_chunks(seed, n, len(wave)):
        ph += O.integrate2_f64_multi(P, pos, mag, im, nr, fp, cc, cubes, grads, wave[t0:t0 + len(d)],
                                     float(pc), d)
    return mag[:, None] * np.exp(1j * ph), pos.reshape(-1, 3)


def run_headline_error(args, W, m):
    """Signal error of the headline workload's FP32 forms against the FP64
    form on the same Philox draws (the FP64 form walks the reference's step in
    double and equals the FP64 oracle bit for bit): every spin of the
    workload over the whole PGSE (delta 15, Delta 40 ms: 11,000 steps)."""
    from dsim_gb300.engine import Batch, Spins, grad_scaled, mesh_run, signal_from_sums
    from dsim_gb300.jobs import fibonacci_dirs, pgse_gmag
    steps = int(round((W.delta + W.Delta) / W.dt))
    nd, nD = int(round(W.delta / W.dt)), int(round(W.Delta / W.dt))
    w = np.zeros(steps, F)
    w[:nd] = 1
    w[nD:nD + nd] = -1
    seed = 5
    t0 = time.time()
    s = Spins(W.N)
    s.set(W.pos, np.ones(W.N, F), np.zeros(W.N, F), W.comp, W.fiber)
    mesh_run(m, s, mesh_params_of(W), grad_per_step=(w[:, None] * W.g[None, :]).astype(F), iterations=steps,
             seed=seed)
    S_plain = signal_from_sums(s.signal())[0]
    assert s.status() == 0
    s.free()
    G = np.concatenate([pgse_gmag(b, W.delta, W.Delta) * fibonacci_dirs(64) for b in (1.0, 2.0, 3.0)])
    gs = np.concatenate([W.g[None, :], grad_scaled(G, W.spaceScale).astype(F).reshape(-1, 3)])
    b = Batch(3 * (W.N + 64), 3)
    sid = b.add_mesh(m)
    common = dict(pos=W.pos, comp=W.comp, fiber=W.fiber.astype(np.uint32), steps=steps, dt=W.dt, step_sd=W.stdDevs,
                  T2=W.T2, phase_constant=W.pc, seed=seed, waveform="pgse", delta=W.delta, Delta=W.Delta)
    j64 = b.submit(sid, precise=True, **common)
    j32 = b.submit(sid, **common)
    jloc = b.submit(sid, local=True, **common)
    b.run()
    st = b.status()
    S = {}
    for name, j in (("fp64", j64), ("batch_fp32", j32), ("local", jloc)):
        sums = b.signal(j, gs)
        S[name] = np.hypot(sums[:, 0, 0], sums[:, 0, 1]) / sums[:, 0, 2]
    b.close()
    return {"workload": "every spin of the headline workload (%d) x %d steps (the whole PGSE), seed %d, the "
                        "headline gradient plus 64 Fibonacci directions x b 1, 2, 3 ms/um2" % (W.N, steps, seed),
            "against": "the FP64 form on the same draws (the reference step in double; equal to the FP64 oracle "
                       "bit for bit)",
            "plain": dict(_err_summary([abs(S_plain - S["fp64"][0])], "FP64 form"),
                          note="the timed form: one walk with the headline gradient (b 3 ms/um2)"),
            "batch_fp32": _err_summary(np.abs(S["batch_fp32"] - S["fp64"]), "FP64 form"),
            "local": _err_summary(np.abs(S["local"] - S["fp64"]), "FP64 form"),
            "signal_headline_fp64": float(S["fp64"][0]), "status": st, "seconds": time.time() - t0}


# --------------------------------------------------------------------------
# batched and served forms on a seeded job mix
# --------------------------------------------------------------------------
def mix_substrates(W, m):
    """The job mixes' substrates, resident for every job: the headline mesh, a
    100-axon mesh, packed cylinders of 64 and 256."""
    from dsim_gb300 import jobs as JB
    return [JB.mesh_substrate(W.axons, 1, mesh=m, tube=W.tube), JB.mesh_substrate(100, 7),
            JB.cyl_substrate(64, 1), JB.cyl_substrate(256, 2)]


def build_mix(W, m, n_jobs, seed, spins_range, steps_range, permeable=False, subs=None):
    from dsim_gb300 import jobs as JB
    t0 = time.time()
    if subs is None:
        subs = mix_substrates(W, m)
    rng = np.random.default_rng(seed)
    mix = [JB.make_job(rng, subs, spins_range=spins_range, steps_range=steps_range, permeable=permeable,
                       seed=1000 + k) for k in range(n_jobs)]
    log("job mix: %d jobs, %.3g spin-steps, %d gradients, built in %.1fs" % (
        n_jobs, sum(j["n"] * j["steps"] for j in mix), sum(len(j["grads"]) for j in mix), time.time() - t0))
    return subs, mix


def _submit_kw(j, form="fp32"):
    """Job keywords; form "fp32": the plain FP32 step with Kahan moments;
    "bar": the forms that hold the 1e-3 signal-error bar (mesh jobs
    and cylinder jobs in the cell-local form, DSIM_JOB_LOCAL); "fp64": the
    step in FP64 (DSIM_JOB_PRECISE)."""
    kw = dict(steps=j["steps"], dt=j["dt"], step_sd=j["step_sd"], T2=j["T2"], phase_constant=j["phase_constant"],
              seed=j["seed"], permeability=j["permeability"], waveform="pgse", delta=j["delta"],
              Delta=j["Delta"], inner_radius_proportion=j["inner"])
    if form == "bar":
        kw.update(local=True)
    elif form == "fp64":
        kw.update(precise=True)
    return kw


def run_plain_mix(mix):
    """One job at a time through the plain path (dsim_mesh_run / dsim_cyl_run),
    one walk with the job's first gradient; host clock from upload to signal.
    Returns the times and the first gradient's signal of every job."""
    from dsim_gb300.engine import Spins, cyl_params, cyl_run, mesh_params, mesh_run, pgse_table
    per, sig0 = [], []
    for k, j in enumerate([mix[0]] + list(mix)):  # the first job once untimed (module load)
        sub = j["sub"]
        w = pgse_table(j["steps"], float(j["dt"]), j["delta"], j["Delta"])
        gps = (w[:, None] * j["grads"][0][None, :]).astype(F)
        s = Spins(j["n"])
        t0 = time.perf_counter()
        if sub.kind == "mesh":
            s.set(j["pos"], np.ones(j["n"], F), np.zeros(j["n"], F), j["comp"], j["fiber"].astype(np.uint16))
            p = mesh_params(j["step_sd"], j["T2"], j["permeability"], j["dt"], j["phase_constant"])
            mesh_run(sub.handle, s, p, grad_per_step=gps, iterations=j["steps"], seed=j["seed"])
        else:
            s.set_cyl(j["pos"], None, None, j["comp"].astype(np.uint32), j["fiber"])
            p = cyl_params(2.0, 2.0, 0.2, sub.spaceScale, 70.0, 8.0, 80.0, j["permeability"], j["inner"],
                           j["dt"], j["phase_constant"])
            cyl_run(sub.handle, s, p, grad_per_step=gps, iterations=j["steps"], seed=j["seed"])
        sums = s.signal()
        if k > 0:
            per.append(time.perf_counter() - t0)
            sig0.append(float(np.hypot(sums[0, 0], sums[0, 1]) / sums[0, 2]))
        del s
    return per, sig0


def run_plain_bar_mix(subs, mix):
    """One job at a time in the forms that hold the 1e-3 error bar (mesh jobs
    and cylinder jobs cell-local): a batch holding that job alone,
    from submission to its first gradient's signal."""
    from dsim_gb300.engine import Batch
    per, sig0 = [], []
    for k, j in enumerate([mix[0]] + list(mix)):  # the first job once untimed (FP64 tables, module load)
        b = Batch((j["n"] + 31) // 32 * 32, 1)
        sid = b.add_mesh(j["sub"].handle) if j["sub"].kind == "mesh" else b.add_cyl(j["sub"].handle)
        t0 = time.perf_counter()
        jid = b.submit(sid, j["pos"], j["comp"], j["fiber"], **_submit_kw(j, "bar"))
        b.run()
        sums = b.signal(jid, j["grads"][:1])[0]
        if k > 0:
            per.append(time.perf_counter() - t0)
            sig0.append(float(np.hypot(sums[0, 0], sums[0, 1]) / sums[0, 2]))
        b.close()
    return per, sig0


def run_batched_mix(subs, mix, cfg, form="fp32"):
    from dsim_gb300.engine import Batch
    cap = sum((j["n"] + 31) // 32 * 32 for j in mix)
    b = Batch(cap, len(mix))
    sids = {id(sb): (b.add_mesh(sb.handle) if sb.kind == "mesh" else b.add_cyl(sb.handle)) for sb in subs}
    b.configure(chunk=cfg["chunk"], occupancy=cfg["occupancy"], graph_chunks=8, block=cfg.get("block"))
    t0 = time.perf_counter()
    ids = [b.submit(sids[id(j["sub"])], j["pos"], j["comp"], j["fiber"], **_submit_kw(j, form)) for j in mix]
    b.run()
    sigs = [b.signal(i, j["grads"]) for i, j in zip(ids, mix)]
    el = time.perf_counter() - t0
    info = b.info()
    st = b.status()
    b.close()
    return el, sigs, info, st


def tune_mix(subs, mix):
    """Autotune on the first jobs of the mix (a separate batch)."""
    from dsim_gb300.engine import Batch
    sample = mix[:8]
    cap = sum((j["n"] + 31) // 32 * 32 for j in sample)
    b = Batch(cap, len(sample))
    sids = {id(sb): (b.add_mesh(sb.handle) if sb.kind == "mesh" else b.add_cyl(sb.handle)) for sb in subs}
    for j in sample:
        b.submit(sids[id(j["sub"])], j["pos"], j["comp"], j["fiber"], **_submit_kw(j))
    best, ms = b.autotune(trial_steps=60)
    b.close()
    return best, ms


SERVE_MAX_CHUNK = 200


def serve_stream(subs, get_job, n_jobs, cfg, rate, form, spin_capacity, seed=3, ahead=0, keep=None):
    """Poisson arrivals at `rate` jobs/s of jobs get_job(0..n_jobs-1) into the
    request loop (150 GB HBM cap).  With `ahead` > 0, host threads generate the
    jobs that many arrivals early and each job's arrays are dropped once it is
    submitted (the server releases its copy on admission).  Returns the
    summary and the signal sums of the jobs in `keep` (all if None)."""
    from concurrent.futures import ThreadPoolExecutor
    from dsim_gb300.engine import Server
    srv = Server(spin_capacity=spin_capacity, job_capacity=n_jobs, hbm_cap=150e9)
    sids = {id(sb): (srv.add_mesh(sb.handle) if sb.kind == "mesh" else srv.add_cyl(sb.handle)) for sb in subs}
    # the server admits at chunk boundaries: at most 200 steps per chunk keeps
    # admission prompt whatever chunk the batch autotuner chose
    srv.configure(chunk=min(cfg["chunk"], SERVE_MAX_CHUNK), occupancy=cfg["occupancy"], graph_chunks=8)
    pool = ThreadPoolExecutor(8) if ahead else None
    futs = {}

    def fetch(k):
        if pool is None:
            return get_job(k)
        for a in range(k, min(n_jobs, k + ahead)):
            if a not in futs:
                futs[a] = pool.submit(get_job, a)
        return futs.pop(k).result()

    if pool is not None:
        # the first window is generated before the clock starts
        for a in range(min(n_jobs, ahead)):
            futs[a] = pool.submit(get_job, a)
        for a in range(min(n_jobs, ahead)):
            futs[a].result()
    srv.start()
    gaps = np.random.default_rng(seed).exponential(1.0 / rate, n_jobs)
    t0 = time.perf_counter()
    tickets, work, late = [], 0.0, 0
    t_next = t0
    for k in range(n_jobs):
        j = fetch(k)
        t_next += gaps[k]
        d = t_next - time.perf_counter()
        if d > 0:
            time.sleep(d)
        elif d < -0.05:
            late += 1
        tickets.append(srv.submit(sids[id(j["sub"])], j["pos"], j["comp"], j["fiber"], j["grads"],
                                  **_submit_kw(j, form)))
        work += j["n"] * j["steps"]
        del j
    srv.drain()
    st = srv.stats()
    srv.stop()
    if pool is not None:
        pool.shutdown()
    lat, first, last, sigs = [], None, None, {}
    for k, t in enumerate(tickets):
        done, sig, tm = srv.poll(t)
        if keep is None or k in keep:
            sigs[k] = sig
        lat.append(tm[2] - tm[0])
        first = tm[0] if first is None else min(first, tm[0])
        last = tm[2] if last is None else max(last, tm[2])
    srv.close()
    return {"rate_jobs_per_s": rate, "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "spin_steps_per_s": work / (last - first), "max_jobs_in_flight": int(st["max_inflight"]),
            "errors": int(st["errors"]), "hbm_peak_GB": st["hbm_peak"] / 1e9, "late_submissions": late,
            "wall_s": last - first, "chunk": min(cfg["chunk"], SERVE_MAX_CHUNK), "spin_capacity": spin_capacity}, sigs


def run_served_mix(subs, mix, cfg, rate, seed=3, form="bar"):
    """Poisson arrivals at `rate` jobs/s of the jobs of `mix` into the request loop."""
    cap = max(sum((j["n"] + 31) // 32 * 32 for j in mix) // 2, max((j["n"] + 31) // 32 * 32 for j in mix))
    o, sigs = serve_stream(subs, mix.__getitem__, len(mix), cfg, rate, form, cap, seed=seed)
    return o, [sigs[k] for k in range(len(mix))]


def run_c4_full(args, W, m):
    """The serving configuration at its full size: a Poisson stream of
    --c4-jobs (2,000) jobs drawn from the batching mix's full ranges (spins
    log-uniform 4k-1M, 2k-10k steps, dt 5-10 us, 6-128 directions x 3
    b-values <= 3000 s/mm2) on the mixes' four resident substrates, permeable
    membranes (per-hit permeation log-uniform 1e-4 - 1e-2), HBM admission cap
    150 GB, at multiples of the plain form's capacity.  Job k comes from its own
    generator seeded (--c4-seed, k), so the stream is fixed.  The plain form
    runs the stream's first --c4-plain-jobs jobs one at a time, in the same
    form; its capacity for the whole stream is the stream's work on each
    substrate over that substrate's plain rate (spin-steps/s of the sample's
    jobs on it), summed, so a sample that holds more of one substrate's work
    than the stream does not bias it.  The signal error against FP64 walks on
    the same draws is taken on --c4-err-jobs jobs spread over the stream."""
    from dsim_gb300 import jobs as JB
    t0 = time.time()
    subs = mix_substrates(W, m)
    n_jobs, seed, form = args.c4_jobs, args.c4_seed, args.c4_form
    spins_range, steps_range = (4096, 1 << 20), (2000, 10000)

    def job(k):
        return JB.make_job(np.random.default_rng([seed, k]), subs, spins_range=spins_range, steps_range=steps_range,
                           permeable=True, seed=100000 + k)

    shapes = [JB.job_shape(np.random.default_rng([seed, k]), subs, spins_range, steps_range) for k in range(n_jobs)]
    work = np.array([float(n) * st for _, n, st in shapes])
    K = min(args.c4_plain_jobs, n_jobs)
    while K < n_jobs and len({id(sb) for sb, _, _ in shapes[:K]}) < len({id(sb) for sb, _, _ in shapes}):
        K += 1                                   # every substrate of the stream in the sample
    sample = [job(k) for k in range(K)]
    best, _ = tune_mix(subs, sample)
    cfg = {"occupancy": best["occupancy"], "chunk": best["chunk"], "block": best.get("block")}
    per = (run_plain_bar_mix(subs, sample) if form == "bar" else run_plain_mix(sample))[0]
    sub_rate = {}
    for sb in {id(sb): sb for sb, _, _ in shapes[:K]}.values():
        ks = [k for k in range(K) if shapes[k][0] is sb]
        sub_rate[id(sb)] = sum(work[k] for k in ks) / sum(per[k] for k in ks)
    plain_s = sum(work[k] / sub_rate[id(shapes[k][0])] for k in range(n_jobs))
    plain_rate = work.sum() / plain_s
    cap_jobs = n_jobs / plain_s
    step = max(1, n_jobs // max(1, args.c4_err_jobs))
    err_ids = list(range(step // 2, n_jobs, step))[:args.c4_err_jobs]
    log("c4 full: %d jobs, %.3g spin-steps, plain %.3g spin-steps/s = %.3f jobs/s; setup %.0f s" % (
        n_jobs, work.sum(), plain_rate, cap_jobs, time.time() - t0))
    out = {"jobs": n_jobs, "seed": seed, "spins": list(spins_range), "steps": list(steps_range),
           "spin_steps": float(work.sum()), "mesh_jobs": int(sum(sb.kind == "mesh" for sb, _, _ in shapes)),
           "permeability": "log-uniform 1e-4 - 1e-2 per hit", "hbm_cap_GB": 150,
           "form": ("cell-local FP32 (DSIM_JOB_LOCAL) for mesh and cylinder jobs"
                    if form == "bar" else "fp32: the plain FP32 step, Kahan moments"),
           "plain": {"spin_steps_per_s": plain_rate, "jobs_per_s": cap_jobs, "sample_jobs": K,
                     "sample_spin_steps_per_s": float(work[:K].sum() / sum(per)),
                     "per_substrate_spin_steps_per_s": [sub_rate.get(id(sb)) for sb in subs],
                     "note": "one job at a time, same form, on the stream's first jobs; the stream's plain time is "
                             "its work on each substrate over that substrate's sample rate"},
           "autotuned": best, "spin_capacity": args.c4_spin_capacity, "rates": []}
    keep = set(err_ids)
    sigs_by_rate = []
    for r in args.c4_rates:
        log("c4 full: rate %.2f x plain (%.3f jobs/s), about %.0f s of arrivals" % (r, r * cap_jobs,
                                                                                    n_jobs / (r * cap_jobs)))
        o, sigs = serve_stream(subs, job, n_jobs, cfg, r * cap_jobs, form, args.c4_spin_capacity, ahead=24,
                               keep=keep)
        o["rate_x_plain_capacity"] = r
        o["speedup_vs_plain"] = o["spin_steps_per_s"] / plain_rate
        out["rates"].append(o)
        sigs_by_rate.append(sigs)
        log("c4 full: %s" % o)
    if err_ids and sigs_by_rate:
        ejobs = [job(k) for k in err_ids]
        ref, cyl_err = mix_fp64_reference(ejobs, ns_cyl=512)
        for o, sigs in zip(out["rates"], sigs_by_rate):
            o["err_vs_fp64"] = mix_err(ejobs, [sigs[k] for k in err_ids], ref, cyl_err)
            o["err_vs_fp64"]["jobs"] = err_ids
    out["seconds"] = time.time() - t0
    return out


def mix_fp64_reference(mix, ns_cyl=2048):
    """FP64 references of a job mix on the same Philox draws.
    Mesh jobs: the FP64 form on the GPU (the reference step in double, equal
    to the FP64 oracle bit for bit), whole jobs: {job: S64 per gradient}.
    Cylinder jobs: the first min(n, ns_cyl) spins as an FP32 batch job and as
    the FP64 oracle walk (oracle/, on the CPU) on the same draws:
    {job: |S32 - S64| per gradient} on that sample."""
    from dsim_gb300.engine import Batch, pgse_table
    mesh = [i for i, j in enumerate(mix) if j["sub"].kind == "mesh"]
    cyl = [i for i, j in enumerate(mix) if j["sub"].kind != "mesh"]
    ref, cyl_err = {}, {}
    if mesh:
        b = Batch(sum((mix[i]["n"] + 31) // 32 * 32 for i in mesh), len(mesh))
        sids = {}
        for i in mesh:
            if id(mix[i]["sub"]) not in sids:
                sids[id(mix[i]["sub"])] = b.add_mesh(mix[i]["sub"].handle)
        ids = {i: b.submit(sids[id(mix[i]["sub"])], mix[i]["pos"], mix[i]["comp"], mix[i]["fiber"], precise=True,
                           **_submit_kw(mix[i])) for i in mesh}
        b.run()
        for i in mesh:
            sums = b.signal(ids[i], mix[i]["grads"])
            ref[i] = np.hypot(sums[:, 0, 0], sums[:, 0, 1]) / sums[:, 0, 2]
        b.close()
    if cyl:
        # cylinder jobs: the precision form on the GPU (the dSim2 step in
        # double, equal to the FP64 oracle bit for bit), whole jobs
        b = Batch(sum((mix[i]["n"] + 31) // 32 * 32 for i in cyl), len(cyl))
        sids = {}
        for i in cyl:
            if id(mix[i]["sub"]) not in sids:
                sids[id(mix[i]["sub"])] = b.add_cyl(mix[i]["sub"].handle)
        ids = {i: b.submit(sids[id(mix[i]["sub"])], mix[i]["pos"], mix[i]["comp"], mix[i]["fiber"], precise=True,
                           **_submit_kw(mix[i])) for i in cyl}
        b.run()
        for i in cyl:
            sums = b.signal(ids[i], mix[i]["grads"])
            ref[i] = np.hypot(sums[:, 0, 0], sums[:, 0, 1]) / sums[:, 0, 2]
        b.close()
        # and the FP64 oracle itself (CPU) on the first spins of the first cylinder job
        i = cyl[0]
        j, n = mix[i], min(mix[i]["n"], ns_cyl)
        b = Batch((n + 31) // 32 * 32, 2)
        sid = b.add_cyl(j["sub"].handle)
        j64 = b.submit(sid, j["pos"][:3 * n], j["comp"][:n], j["fiber"][:n], precise=True, **_submit_kw(j))
        b.run()
        _, bmag, bmom, _, _ = b.get(j64, n)
        b.close()
        ss = F(j["sub"].spaceScale)
        adc = tuple(F(a) / (ss * ss) for a in (2.0, 0.2, 2.0))      # intra, myelin, extra (jobs.make_job)
        wave = pgse_table(j["steps"], float(j["dt"]), j["delta"], j["Delta"])
        z64, _ = cyl_fp64_z(j["sub"].handle, j["pos"][:3 * n], j["comp"][:n], j["fiber"][:n], adc, j["T2"],
                            j["permeability"], j["inner"], j["dt"], j["phase_constant"], j["grads"], wave, j["seed"])
        cyl_err["oracle_check_max_abs_dS"] = float(np.max(np.abs(_S(_z_from_moments(bmag, bmom, j["grads"],
                                                                                     j["phase_constant"])) - _S(z64))))
    return ref, cyl_err


def mix_err(mix, sigs, ref, cyl_err):
    """A form's error summary: every job's signals `sigs` (sums [nG][5][3]) against
    the FP64 references of mix_fp64_reference (whole jobs, same draws)."""
    d = {i: np.abs(np.hypot(sigs[i][:, 0, 0], sigs[i][:, 0, 1]) / sigs[i][:, 0, 2] - ref[i]) for i in ref}
    me = [d[i] for i in d if mix[i]["sub"].kind == "mesh"]
    ce = [d[i] for i in d if mix[i]["sub"].kind != "mesh"]
    out = {"all": _err_summary(np.concatenate(me + ce), "FP64 on the same Philox draws, whole jobs")}
    if me:
        out["mesh_jobs"] = _err_summary(np.concatenate(me), "the FP64 form (equal to the FP64 oracle bit for bit)")
    if ce:
        out["cylinder_jobs"] = _err_summary(np.concatenate(ce), "the FP64 form (equal to the FP64 oracle bit for "
                                                                 "bit)")
    if "oracle_check_max_abs_dS" in cyl_err:
        out["cylinder_fp64_form_vs_oracle_max_abs_dS"] = cyl_err["oracle_check_max_abs_dS"]
    return out


def run_forms(args, W, m):
    n_jobs = args.mix_jobs
    spins_range = (4096, args.mix_max_spins)
    steps_range = (args.mix_min_steps, args.mix_max_steps)
    subs, mix = build_mix(W, m, n_jobs, 11, spins_range, steps_range)
    work = sum(j["n"] * j["steps"] for j in mix)
    grad_work = sum(j["n"] * j["steps"] * len(j["grads"]) for j in mix)
    if args.mix_config:
        occ, chunk = args.mix_config
        best = {"occupancy": occ, "chunk": chunk, "fine_per_ref": None, "block": args.mix_block, "fixed": True}
    else:
        best, tune_ms = tune_mix(subs, mix)
        log("autotune: %s (%.1f ms for 60 steps of 8 jobs)" % (best, tune_ms))
    cfg = {"occupancy": best["occupancy"], "chunk": best["chunk"], "block": best.get("block")}
    per, psig = run_plain_mix(mix)
    plain_s = sum(per)
    per_b, bsig = run_plain_bar_mix(subs, mix)
    plainbar_s = sum(per_b)
    el, sigs, info, st = run_batched_mix(subs, mix, cfg)
    plain_rate = work / plain_s
    plainbar_rate = work / plainbar_s
    t_err = time.time()
    ref, cyl_err = mix_fp64_reference(mix)
    batched_err = mix_err(mix, sigs, ref, cyl_err)
    batched_err["seconds"] = time.time() - t_err
    first = lambda v: [np.array([[[x, 0.0, 1.0]] + [[0.0, 0.0, 0.0]] * 4]) for x in v]   # S as sums (X, Y=0, n=1)
    out = {
        "mix": {"jobs": n_jobs, "spins": list(spins_range), "steps": list(steps_range), "dt_us": [5, 10],
                "substrates": "beaded tubes 400 and 100 axons (2.56M / 0.64M triangles), packed cylinders 64 and 256",
                "gradients_per_job": "6-128 directions x 3 b-values (b <= 3000 s/mm2), one PGSE waveform",
                "spin_steps": work},
        "plain": {"spin_steps_per_s": plain_rate, "seconds": plain_s,
                  "err_vs_fp64": mix_err(mix, first(psig), {i: r[:1] for i, r in ref.items()}, {}),
                  "note": "one job at a time (dsim_mesh_run / dsim_cyl_run), one walk per job with its first "
                          "gradient; the reference's FP32 step"},
        "plain_bar": {"spin_steps_per_s": plainbar_rate, "seconds": plainbar_s,
                      "err_vs_fp64": mix_err(mix, first(bsig), {i: r[:1] for i, r in ref.items()}, {}),
                      "note": "one job at a time in the forms that hold the 1e-3 bar (a batch holding that job "
                              "alone: cell-local mesh and cylinder jobs), first gradient"},
        "batched": {"spin_steps_per_s": work / el, "seconds": el, "speedup_vs_plain": (work / el) / plain_rate,
                    "signals_speedup_vs_plain": (grad_work / el) / plain_rate,
                    "note": "all jobs in one batch; signals_speedup counts one plain walk per gradient, as the "
                            "reference re-walks every gradient",
                    "autotuned": best, "kernel_launches": info["launches"], "graph_launches": info["graph_launches"],
                    "status": st, "err_vs_fp64": batched_err, "form": "fp32: the plain FP32 step, Kahan moments"},
    }
    # the same mix in the forms that hold the 1e-3 error bar
    el_b, sigs_b, info_b, st_b = run_batched_mix(subs, mix, cfg, form="bar")
    out["batched_bar"] = {"spin_steps_per_s": work / el_b, "seconds": el_b,
                          "speedup_vs_plain_bar": (work / el_b) / plainbar_rate,
                          "speedup_vs_plain": (work / el_b) / plain_rate,
                          "signals_speedup_vs_plain_bar": (grad_work / el_b) / plainbar_rate,
                          "status": st_b, "err_vs_fp64": mix_err(mix, sigs_b, ref, cyl_err),
                          "form": "cell-local FP32 (DSIM_JOB_LOCAL) for mesh and cylinder jobs"}
    # serving: the same substrates and ranges with permeable membranes (per-hit
    # permeation log-uniform 1e-4 - 1e-2), in the error-bar forms; arrival
    # rates relative to the capacity of the plain form at the same bar (one
    # job at a time) on that mix
    out["served"] = []
    if args.serve_rates:
        _, pmix = build_mix(W, m, n_jobs, 12, spins_range, steps_range, permeable=True, subs=subs)
        pwork = sum(j["n"] * j["steps"] for j in pmix)
        pplain_s = sum(run_plain_mix(pmix)[0])
        pbar_s = sum(run_plain_bar_mix(subs, pmix)[0])
        cap_jobs = n_jobs / pbar_s
        out["served_mix"] = {"jobs": n_jobs, "seed": 12, "permeability": "log-uniform 1e-4 - 1e-2 per hit",
                             "plain_spin_steps_per_s": pwork / pplain_s, "plain_jobs_per_s": n_jobs / pplain_s,
                             "plain_bar_spin_steps_per_s": pwork / pbar_s, "plain_bar_jobs_per_s": cap_jobs,
                             "rates_relative_to": "plain_bar_jobs_per_s"}
        pref, pcyl = mix_fp64_reference(pmix)
        for r in args.serve_rates:
            o, ssig = run_served_mix(subs, pmix, cfg, r * cap_jobs)
            o["rate_x_plain_bar_capacity"] = r
            o["speedup_vs_plain_bar"] = o["spin_steps_per_s"] / (pwork / pbar_s)
            o["err_vs_fp64"] = mix_err(pmix, ssig, pref, pcyl)
            o["form"] = "cell-local FP32 (DSIM_JOB_LOCAL) for mesh and cylinder jobs"
            out["served"].append(o)
    return out


# --------------------------------------------------------------------------
# cylinders (C1): 64 z-cylinders, 10k spins, 5000 steps, 48 PGSE gradients
# --------------------------------------------------------------------------
def run_cylinders(args):
    from dsim_gb300 import jobs as JB
    from dsim_gb300.engine import Batch, Spins, cyl_params, cyl_run, grad_scaled, pgse_table, phase_constant
    sub = JB.cyl_substrate(64, 1)          # 20 x 20 um cell, spaceScale 10
    c = sub.handle
    N, dt, steps, delta, Delta = args.c1_spins, 0.01, args.c1_steps, 10.0, 30.0
    rng = np.random.default_rng(1)
    pos = rng.uniform(-0.995, 0.995, (N, 3)).astype(F)
    imo, near = JB.cyl_regions(sub.geom, pos, sub.spaceScale)
    dirs = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0], [1, 0, 1], [0, 1, 1]], np.float64)
    dirs /= np.linalg.norm(dirs, axis=1)[:, None]
    G = np.concatenate([lv * dirs for lv in np.linspace(0.0, 80.0, 8)])          # 48 x 3, mT/m
    gs = grad_scaled(G, sub.spaceScale).astype(F).reshape(-1, 3)
    pc = phase_constant(42576.0, dt)
    w = pgse_table(steps, dt, delta, Delta)
    ss = F(sub.spaceScale)
    sd = [float(np.sqrt(F(2) * (F(adc) / (ss * ss)) * F(dt))) for adc in (2.0, 2.0, 2.0)] + [0.0]
    T2 = [0.0, 0.0, 0.0, 0.0]                                               # no T2 decay in C1
    # plain path: one fresh walk per gradient, one after another (the reference's order)
    p = cyl_params(2.0, 2.0, 2.0, sub.spaceScale, 1e30, 1e30, 1e30, 0.0, 1.0, dt, pc)
    s = Spins(N)
    s.set_cyl(pos, None, None, imo.astype(np.uint32), near)
    cyl_run(c, s, p, grad_per_step=(w[:, None] * gs[0][None, :]).astype(F), iterations=50, seed=99)
    s.sync()
    t0 = time.perf_counter()
    plain_S = []
    for k, g in enumerate(gs):
        s.set_cyl(pos, None, None, imo.astype(np.uint32), near)
        cyl_run(c, s, p, grad_per_step=(w[:, None] * g[None, :]).astype(F), iterations=steps, seed=k + 1)
        sums = s.signal(0.8)                      # dSim2 reads spins inside +-0.8
        plain_S.append(float(np.hypot(sums[0, 0], sums[0, 1]) / sums[0, 2]))
    plain_s = time.perf_counter() - t0
    # batch form: the same 48 fresh walks as 48 jobs of one launch
    b = Batch(48 * ((N + 31) // 32 * 32), 48)
    sid = b.add_cyl(c)
    t0 = time.perf_counter()
    ids = [b.submit(sid, pos.reshape(-1), imo, near, steps, dt, sd, T2, pc, k + 1, waveform="pgse", delta=delta,
                    Delta=Delta, inner_radius_proportion=1.0) for k in range(len(gs))]
    b.run()
    batch_S = []
    for k, j in enumerate(ids):
        sums = b.signal(j, gs[k][None, :], region=0.8)[0]
        batch_S.append(float(np.hypot(sums[0, 0], sums[0, 1]) / sums[0, 2]))
    batch_s = time.perf_counter() - t0
    counts = b.counts(ids[0])
    b.close()
    # one shared walk: every gradient from the moments of a single walk
    b = Batch((N + 31) // 32 * 32, 1)
    sid = b.add_cyl(c)
    t0 = time.perf_counter()
    j = b.submit(sid, pos.reshape(-1), imo, near, steps, dt, sd, T2, pc, 1, waveform="pgse", delta=delta,
                 Delta=Delta, inner_radius_proportion=1.0)
    b.run()
    sums = b.signal(j, gs, region=0.8)
    shared_S = (np.hypot(sums[:, 0, 0], sums[:, 0, 1]) / sums[:, 0, 2]).tolist()
    shared_s = time.perf_counter() - t0
    sw_pos, sw_mag, sw_mom, _, _ = b.get(j, N)
    b.close()
    # signal error against the FP64 oracle walk on the same Philox draws
    t_err = time.perf_counter()
    in_box = lambda q: np.all(np.abs(np.asarray(q).reshape(-1, 3)) < 0.8, axis=1)
    adc = (F(2.0) / (ss * ss),) * 3
    z64, p64 = cyl_fp64_z(c, pos, imo, near, adc, [0, 0, 0], 0.0, 1.0, dt, pc, gs, w, 1)
    z32 = _z_from_moments(sw_mag, sw_mom, gs, pc)
    err_shared = np.abs(_S(z32, in_box(sw_pos)) - _S(z64, in_box(p64)))
    err_plain = []
    for k in range(len(gs) - 6, len(gs)):          # 80 mT/m along each of the 6 directions
        zk, pk = cyl_fp64_z(c, pos, imo, near, adc, [0, 0, 0], 0.0, 1.0, dt, pc, gs[k][None, :], w, k + 1)
        err_plain.append(abs(plain_S[k] - float(_S(zk, in_box(pk))[0])))
    # the shared walk in the cylinder precision form (FP64 positions)
    b = Batch((N + 31) // 32 * 32, 1)
    sid = b.add_cyl(c)
    t0 = time.perf_counter()
    j = b.submit(sid, pos.reshape(-1), imo, near, steps, dt, sd, T2, pc, 1, waveform="pgse", delta=delta,
                 Delta=Delta, inner_radius_proportion=1.0, precise=True)
    b.run()
    sums = b.signal(j, gs, region=0.8)
    prec_s = time.perf_counter() - t0
    S_prec = np.hypot(sums[:, 0, 0], sums[:, 0, 1]) / sums[:, 0, 2]
    b.close()
    # and in the cylinder cell-local form
    b = Batch((N + 31) // 32 * 32, 1)
    sid = b.add_cyl(c)
    t0 = time.perf_counter()
    j = b.submit(sid, pos.reshape(-1), imo, near, steps, dt, sd, T2, pc, 1, waveform="pgse", delta=delta,
                 Delta=Delta, inner_radius_proportion=1.0, local=True)
    b.run()
    sums = b.signal(j, gs, region=0.8)
    loc_s = time.perf_counter() - t0
    S_loc = np.hypot(sums[:, 0, 0], sums[:, 0, 1]) / sums[:, 0, 2]
    loc_tests, loc_exact = b.precision_counts(j)
    b.close()
    err = {"shared_walk": _err_summary(err_shared, "FP64 oracle walk on the same Philox draws, all 48 gradients"),
           "shared_walk_precise": dict(_err_summary(np.abs(S_prec - _S(z64, in_box(p64))), "FP64 oracle walk on "
                                                    "the same Philox draws, all 48 gradients"),
                                       form="DSIM_JOB_PRECISE: the dSim2 step with FP64 positions",
                                       spin_steps_per_s=N * steps / prec_s),
           "shared_walk_local": dict(_err_summary(np.abs(S_loc - _S(z64, in_box(p64))), "FP64 oracle walk on "
                                                  "the same Philox draws, all 48 gradients"),
                                     form="DSIM_JOB_LOCAL: the dSim2 step on FP32 offsets from a 1/16 lattice, "
                                          "FP64 decisions inside the FP32 error band",
                                     spin_steps_per_s=N * steps / loc_s,
                                     fp64_decision_fraction=loc_exact / max(loc_tests, 1)),
           "plain": _err_summary(err_plain, "FP64 oracle walk on each walk's Philox draws, 80 mT/m along the "
                                            "6 directions"),
           "seconds": time.perf_counter() - t_err}
    # C-bar: cell-list entries a step examines (own fiber inside; the new
    # position's cell list outside), from the initial state
    cc, cubes, fp = c.grid()
    n3 = c.numCubes
    cell = np.clip(np.floor((pos.astype(np.float64) + 1.0) / float(c.cubeLength)), 0, n3 - 1).astype(np.int64)
    key = cell[:, 2] * n3 * n3 + cell[:, 1] * n3 + cell[:, 0]
    Cbar = float(np.where(imo < 2, 1.0, cc[key].astype(np.float64)).mean())
    work = len(gs) * N * steps
    res = {"workload": "64 z-cylinders (Gamma radii mean 1 um, 0.5 packing, 20 x 20 um, spaceScale 10), %d spins, "
                       "dt 10 us, %d steps, PGSE delta 10 Delta 30 ms, 8 levels 0-80 mT/m x 6 directions" % (N, steps),
           "boundary": "clamped box (the reference has no periodic boundaries)",
           "plain_spin_steps_per_s": work / plain_s, "batched_spin_steps_per_s": work / batch_s,
           "shared_walk_signals_per_s": len(gs) / shared_s, "shared_walk_seconds": shared_s,
           "plain_seconds": plain_s, "batched_seconds": batch_s,
           "signal_plain": plain_S[::8], "signal_batched": batch_S[::8], "signal_shared_walk": shared_S[::8],
           "rejections_per_spin_step": float(counts[0]) / (N * steps),
           "err_vs_fp64": err, "readout": "spins inside +-0.8 (dSim2 getMrSignal)",
           "roofline": {"bytes_per_spin_step": 2 * 20 + 16 * Cbar, "C_bar": Cbar,
                        "achieved_GBs_batched": (2 * 20 + 16 * Cbar) * work / batch_s / 1e9,
                        "fine_grid": c.fine_info(),
                        "note": "bytes of the reference's scan (C_bar list entries a step examines); the fine "
                                "filter grid tests only the entries of the spin's fine cell (about 2 here), with "
                                "equal results, so achieved can exceed the HBM copy peak: the kernel reads its "
                                "fibers and grid from L1/L2 and is bound by instruction issue"},
           "note": "signals listed for every 8th gradient (G = 0 .. 80 mT/m along x)"}
    # the reference's CPU path (oracle port, MWC draws) on a sample
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    P = O.Params2()
    P.intraAdcScaled = P.extraAdcScaled = P.myelinAdcScaled = F(2.0) / (ss * ss)
    P.T2fiber = P.T2myelin = P.T2outside = 1e30
    P.permeability, P.innerRadiusProportion, P.spinRadius, P.deltaTime = 0.0, 1.0, 0.005, dt
    P.numCubes, P.maxFibersPerCube, P.cubeLength = c.numCubes, c.maxFPC, c.cubeLength
    ns, it = 2000, 400
    p4 = np.zeros((ns, 4), F); p4[:, :3] = pos[:ns]
    sd4 = np.zeros((ns, 4), np.uint32)
    sd4[:, :2] = rng.integers(1, 2 ** 31, (ns, 2))
    par = np.zeros((ns, 5), F); par[:, 0] = 1.0
    par[:, 2] = np.where(imo[:ns] < 2, near[:ns], 0).astype(F); par[:, 3] = imo[:ns].astype(F)
    t0 = time.perf_counter()
    O.lib().or2_integrate(C.byref(P), ns, p4.reshape(-1), sd4.reshape(-1), par.reshape(-1), fp, cc, cubes,
                          float(gs[-1][0]), float(gs[-1][1]), float(gs[-1][2]), float(pc), it, None, None, None)
    res["cpu_port_spin_steps_per_s"] = ns * it / (time.perf_counter() - t0)
    res["cpu_port_sample"] = "%d spins x %d steps, 1 thread, the reference's MWC draws" % (ns, it)
    return res


# --------------------------------------------------------------------------
# precision form (C5): the FP64 step vs the FP64 oracle, the plain FP32 form beside it
# --------------------------------------------------------------------------
def c5_waves(steps, dt):
    """PGSE (delta 10, Delta 25 ms scaled into the walk) and 8 OGSE cosines
    of 50-200 Hz over the same gradient windows."""
    from dsim_gb300.engine import pgse_table
    T = steps * dt
    delta, Delta = 0.4 * T, 0.55 * T
    w = [pgse_table(steps, dt, delta, Delta)]
    nd, nD = int(round(delta / dt)), int(round(Delta / dt))
    t = np.arange(steps) * dt
    freqs = np.linspace(50.0, 200.0, 8)
    for f in freqs:
        x = np.zeros(steps)
        x[:nd] = np.cos(2 * np.pi * f * 1e-3 * t[:nd])
        x[nD:nD + nd] = -np.cos(2 * np.pi * f * 1e-3 * (t[nD:nD + nd] - t[nD]))
        w.append(x.astype(F))
    return np.array(w, F), delta, Delta, freqs


def run_precision(args, W, m):
    from dsim_gb300.engine import Batch, grad_scaled, phase_constant, rng_draws, std_devs
    from dsim_gb300.jobs import fibonacci_dirs, pgse_gmag
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    dt = 0.002
    steps = args.c5_steps
    n = args.c5_sample
    waves, delta, Delta, freqs = c5_waves(steps, dt)
    sd = std_devs(W.D, W.D, 0.1 * W.D, W.spaceScale, dt)
    pc = phase_constant(42576.0, dt)
    sel = np.random.default_rng(9).choice(W.N, n, replace=False)
    pos0 = W.pos.reshape(-1, 3)[sel].reshape(-1).copy()
    comp0, fib0 = W.comp[sel].copy(), W.fiber[sel].astype(np.uint32)
    seed = 77
    b = Batch(1 << 16, 3 * len(waves))
    sid = b.add_mesh(m)
    common = dict(pos=pos0, comp=comp0, fiber=fib0, steps=steps, dt=dt, step_sd=sd, T2=W.T2, phase_constant=pc,
                  seed=seed, waveform="table")
    t0 = time.time()
    prec = [b.submit(sid, table=w, precise=True, **common) for w in waves]
    local = [b.submit(sid, table=w, local=True, **common) for w in waves]
    plain = [b.submit(sid, table=w, precise=False, **common) for w in waves]
    b.run()
    gpu_s = time.time() - t0
    # FP64 oracle on the same spins and draws (grid as the reference builds it)
    t0 = time.time()
    d = np.stack([rng_draws(seed, 0, s, n) for s in range(steps)])
    start, tri = m.grid()
    counts = np.diff(start.astype(np.int64)).astype(np.uint32)
    maxtpc = int(counts.max())
    dense = np.zeros((len(counts), maxtpc), np.uint32)
    idx = np.repeat(np.arange(len(counts)), counts)
    off = np.arange(len(tri)) - np.repeat(start[:-1].astype(np.int64), counts)
    dense[idx, off] = tri
    v, ti = m.arrays()
    p = O.params3(sd, W.T2, 0.0, dt, W.numCubes, maxtpc)
    pos = pos0.astype(np.float64)
    mag = np.ones(n, np.float64)
    comp, fib = comp0.copy(), fib0.astype(np.uint16)
    capped, M64 = O.integrate3_f64_moments(p, pos, mag, comp, fib, v, W.tube["trgls"].reshape(-1), ti, counts,
                                           dense.reshape(-1), waves.astype(np.float64), d,
                                           nthreads=os.cpu_count() or 1)
    oracle_s = time.time() - t0
    dirs = fibonacci_dirs(32)
    bvals = [1.0, 3.0, 5.0, 10.0]
    err = {"precise": [], "local": [], "plain": []}
    rms_dz = {"precise": [], "local": [], "plain": []}
    diverged = {}
    exact_pos = True
    for k in range(len(waves)):
        for form, ids in (("precise", prec), ("local", local), ("plain", plain)):
            bpos, bmag, mom, _, _ = b.get(ids[k], n)
            if form != "plain":
                bpos, bmag = b.get_precise(ids[k], n)
            if form == "precise":
                exact_pos &= bool(np.array_equal(bpos.reshape(-1).view(np.uint64), pos.view(np.uint64)))
            if k == 0:
                dp = np.abs(bpos.reshape(-1, 3).astype(np.float64) - pos.reshape(-1, 3)).max(1)
                diverged[form] = float((dp > 1e-4).mean())
            M32 = mom[:, :3].astype(np.float64) - mom[:, 3:].astype(np.float64)
            for bv in bvals:
                gm = min(pgse_gmag(bv, delta, Delta), 300.0)   # |G| <= 300 mT/m
                gs = grad_scaled(gm * dirs, W.spaceScale).astype(np.float64)
                z32 = bmag[:, None] * np.exp(1j * float(pc) * (M32 @ gs.T))
                z64 = mag[:, None] * np.exp(1j * float(pc) * (M64[:, k, :] @ gs.T))
                S32 = np.abs(np.sum(z32, 0)) / n
                S64 = np.abs(np.sum(z64, 0)) / n
                err[form].extend(np.abs(S32 - S64).tolist())
                rms_dz[form].extend(np.sqrt(np.mean(np.abs(z32 - z64) ** 2, 0)).tolist())
    records, exact = b.precision_counts(prec[0])
    l_records, l_retests = b.precision_counts(local[0])
    b.close()
    # throughput of the precision form vs the plain form at full spin count
    rates = {}
    for form in ("plain", "local", "precise"):
        bb = Batch(W.N + 64, 1)
        sid = bb.add_mesh(m)
        jid = bb.submit(sid, W.pos, W.comp, W.fiber.astype(np.uint32), args.c5_rate_steps, dt, sd, W.T2, pc, 5,
                        waveform="table", table=np.resize(waves[1], args.c5_rate_steps).astype(F),
                        precise=(form == "precise"),
                        local=(form == "local"))
        bb.sync()
        t0 = time.time()
        bb.run()
        rates[form] = W.N * args.c5_rate_steps / (time.time() - t0)
        bb.close()
    return {"sample": "%d spins x %d steps at dt 2 us of the 2.56M-triangle mesh, 9 waveforms (PGSE + OGSE %s Hz) "
                      "x 32 directions x b %s ms/um2 (|G| <= 300 mT/m)" % (n, steps, [int(f) for f in freqs], bvals),
            "max_abs_dS_precise": float(np.max(err["precise"])), "median_abs_dS_precise": float(np.median(err["precise"])),
            "max_abs_dS_plain": float(np.max(err["plain"])), "median_abs_dS_plain": float(np.median(err["plain"])),
            "max_abs_dS_local": float(np.max(err["local"])), "median_abs_dS_local": float(np.median(err["local"])),
            "spins_diverged_precise": diverged["precise"], "spins_diverged_plain": diverged["plain"],
            "spins_diverged_local": diverged["local"],
            "max_abs_dS_at_full_spins_precise": float(np.max(rms_dz["precise"])) / np.sqrt(W.N),
            "max_abs_dS_at_full_spins_plain": float(np.max(rms_dz["plain"])) / np.sqrt(W.N),
            "max_abs_dS_at_full_spins_local": float(np.max(rms_dz["local"])) / np.sqrt(W.N),
            "positions_bit_exact_precise": exact_pos,
            "dS_note": ("the precision form walks the FP64 algorithm (positions equal the FP64 oracle's bit for bit; "
                        "|dS| is rounding of the stored moments); the plain form's |dS| is set by the few spins whose "
                        "FP32 path parts from the FP64 one (final position > 1e-4 apart); those differences are "
                        "zero-mean, so at the full spin count the expected |dS| is rms(z - z64) / sqrt(N), reported "
                        "per gradient as max over gradients"),
            "fp64_test_fraction": exact / max(records, 1), "records_examined": records, "fp64_tests": exact,
            "local_fp64_retest_fraction": l_retests / max(l_records, 1),
            "forms": {"precise": "the step in FP64 (DSIM_JOB_PRECISE)",
                      "local": "FP32 offsets from a 1/16 lattice, FP64 re-tests of near-degenerate intersections, "
                               "Kahan moments (DSIM_JOB_LOCAL)",
                      "plain": "the reference's FP32 step with Kahan moments"},
            "spin_steps_per_s_precise": rates["precise"], "spin_steps_per_s_plain_batch": rates["plain"],
            "spin_steps_per_s_local": rates["local"],
            "rate_workload": "%d spins x %d steps, one job" % (W.N, args.c5_rate_steps),
            "gpu_s": gpu_s, "oracle_s": oracle_s, "oracle": "FP64 restatement of the reference step (oracle), same draws"}


def run_precision_full(args, W, m):
    """C5 at full size: every spin of the workload, 20,000 steps at dt 2 us,
    PGSE and OGSE 50 / 200 Hz, in the three forms.  The FP64 form (bit-exact
    with the FP64 oracle on samples) is the reference; per-gradient |dS| of
    the cell-local and plain forms against it over 32 directions x b."""
    from dsim_gb300.engine import Batch, grad_scaled, phase_constant, std_devs
    from dsim_gb300.jobs import fibonacci_dirs, pgse_gmag
    dt = 0.002
    steps = args.c5_steps
    waves, delta, Delta, freqs = c5_waves(steps, dt)
    waves = waves[[0, 1, len(waves) - 1]]  # PGSE, OGSE 50 Hz, OGSE 200 Hz
    sd = std_devs(W.D, W.D, 0.1 * W.D, W.spaceScale, dt)
    pc = phase_constant(42576.0, dt)
    dirs = fibonacci_dirs(32)
    bvals = [1.0, 3.0, 5.0, 10.0]
    gs = np.concatenate([grad_scaled(min(pgse_gmag(bv, delta, Delta), 300.0) * dirs, W.spaceScale)
                         for bv in bvals]).astype(F)
    out = {"workload": "%d spins x %d steps at dt 2 us, waveforms PGSE and OGSE 50 / 200 Hz, 32 directions x b %s "
                       "ms/um2 (|G| <= 300 mT/m)" % (W.N, steps, bvals)}
    sig = {}
    for form in ("precise", "local", "plain"):
        b = Batch(len(waves) * (W.N + 32), len(waves))
        sid = b.add_mesh(m)
        t0 = time.time()
        ids = [b.submit(sid, W.pos, W.comp, W.fiber.astype(np.uint32), steps, dt, sd, W.T2, pc, 77,
                        waveform="table", table=w, precise=(form == "precise"), local=(form == "local"))
               for w in waves]
        b.run()
        b.sync()
        el = time.time() - t0
        assert b.status() in (0, 1)
        sig[form] = np.stack([b.signal(j, gs) for j in ids])  # [wave][grad][5][3]
        out["spin_steps_per_s_" + form] = len(waves) * W.N * steps / el
        out["status_" + form] = int(b.status())
        b.close()
    S = {k: np.hypot(v[:, :, 0, 0], v[:, :, 0, 1]) / v[:, :, 0, 2] for k, v in sig.items()}
    for form in ("local", "plain"):
        d = np.abs(S[form] - S["precise"])
        out["max_abs_dS_" + form] = float(d.max())
        out["median_abs_dS_" + form] = float(np.median(d))
    out["reference"] = "the FP64 form (DSIM_JOB_PRECISE), bit-exact with the FP64 oracle on samples"
    return out


# --------------------------------------------------------------------------
def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--axons", type=int, default=400)
    ap.add_argument("--spins", type=int, default=1 << 20)
    ap.add_argument("--steps-per-launch", type=int, default=1000)
    ap.add_argument("--accel", type=int, default=-1, help="fine grid cells per axis (-1: the default, 2.25 per reference cell)")
    ap.add_argument("--sort-every", type=int, default=-1, help="steps between spin reorderings (-1 default)")
    ap.add_argument("--kernel", type=int, default=0, help="step kernel variant (0 default)")
    ap.add_argument("--records", type=int, default=0, help="fine-grid record bytes (0 default)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-err", action="store_true", help="skip the headline signal error against the FP64 form")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the batched / served job-mix runs")
    ap.add_argument("--mix-jobs", type=int, default=48)
    ap.add_argument("--mix-max-spins", type=int, default=1 << 18)
    ap.add_argument("--mix-min-steps", type=int, default=400)
    ap.add_argument("--mix-max-steps", type=int, default=2000)
    ap.add_argument("--serve-rates", type=float, nargs="*", default=[0.5, 1.0, 1.5, 3.0])
    ap.add_argument("--mix-config", type=int, nargs=2, default=None, metavar=("OCCUPANCY", "CHUNK"),
                    help="fixed batch occupancy and chunk for the job mix instead of autotuning")
    ap.add_argument("--no-precision", action="store_true", help="skip the precision-form comparison")
    ap.add_argument("--no-cylinders", action="store_true", help="skip the cylinder workload")
    ap.add_argument("--c1-spins", type=int, default=10000)
    ap.add_argument("--c1-steps", type=int, default=5000)
    ap.add_argument("--c5-steps", type=int, default=20000)
    ap.add_argument("--c5-sample", type=int, default=512)
    ap.add_argument("--c5-rate-steps", type=int, default=2000)
    ap.add_argument("--no-c5-full", action="store_true",
                    help="skip the full-size precision comparison that a one-GPU run does by default")
    ap.add_argument("--c5-full", action="store_true",
                    help="also run the precision comparison at full size (every spin, --c5-steps steps, 3 waveforms)")
    ap.add_argument("--mix-block", type=int, default=None, choices=[64, 128, 256],
                    help="block size of the plain batch step kernels with --mix-config")
    ap.add_argument("--mix-only", choices=["fp32", "bar", "fp64"], default=None,
                    help="only run the 48-job mix once in one batch in this form (for profiling)")
    ap.add_argument("--c4-full", action="store_true",
                    help="also run the serving configuration at full size (--c4-jobs Poisson jobs of the full "
                         "batching ranges, permeable, 150 GB cap, at --c4-rates x the plain capacity)")
    ap.add_argument("--c4-jobs", type=int, default=2000)
    ap.add_argument("--c4-rates", type=float, nargs="+", default=[0.5, 1.0, 1.5])
    ap.add_argument("--c4-form", default="fp32", choices=["fp32", "bar"])
    ap.add_argument("--c4-seed", type=int, default=13)
    ap.add_argument("--c4-plain-jobs", type=int, default=48)
    ap.add_argument("--c4-err-jobs", type=int, default=8)
    ap.add_argument("--c4-spin-capacity", type=int, default=1 << 22,
                    help="server spin slots: enough to fill the GPU; more slots slow every admitted job")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        import ctypes
        # one GPU per rank
        os.environ["CUDA_VISIBLE_DEVICES"] = os.environ.get("LOCAL_RANK", "0")
    if args.mix_only:
        res = run_mix_only(args) if rank == 0 else None
    else:
        res = run_reference(args, rank, world) if args.impl == "reference" else run_ours(args, rank, world)
    if rank == 0 and res is not None:
        print(json.dumps(res))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
