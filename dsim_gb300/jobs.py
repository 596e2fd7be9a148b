"""Seeded job mixes for the batching and serving forms.

A job is one diffusion simulation: a substrate (beaded-tube mesh or packed
cylinders), a spin count, a step count and time step, and a gradient table
(directions x b-values sharing one PGSE waveform).  The reference simulates
each gradient with a fresh walk (dSim3/src/diffusion.cpp:553-625); the batch
form walks once per job and evaluates every gradient from the spins' gradient
moments.  Substrates are built once and shared by many jobs, as a serving
system keeps them resident.
"""
import math

import numpy as np

from . import substrates as S
from .engine import Cylinders, Mesh, grad_scaled, phase_constant, std_devs

F = np.float32
GAMMA = 42576.0  # kHz/T (the reference's sim.cfg gamma for protons)


def fibonacci_dirs(n):
    """n unit vectors on a Fibonacci sphere (half-integer offsets)."""
    k = np.arange(n) + 0.5
    z = 1 - 2 * k / n
    r = np.sqrt(1 - z * z)
    phi = np.pi * (3 - np.sqrt(5)) * k
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], 1)


def pgse_gmag(b, delta, Delta, gamma=GAMMA):
    """|G| in mT/m for b (ms/um^2) with PGSE delta, Delta (ms):
    b = (2 pi gamma G delta)^2 (Delta - delta/3), gamma in kHz/T."""
    return math.sqrt(b / (Delta - delta / 3.0)) / (2 * math.pi * gamma * 1e-9 * delta)


class Substrate:
    def __init__(self, kind, handle, spaceScale, geom):
        self.kind, self.handle, self.spaceScale, self.geom = kind, handle, spaceScale, geom


def mesh_substrate(axons, seed, mesh=None, tube=None):
    """Beaded tubes in a 50 um cube (spaceScale 25, 1 um reference cells)."""
    if tube is None:
        tube = S.beaded_tubes(n_axons=axons, verts_per_ring=32, ring_spacing=0.5, length=50.0, box=50.0,
                              seed=seed, membranes="G", allow_overlap=True)
    if mesh is None:
        mesh = Mesh.from_arrays(tube["vertices"], tube["trgls"], tube["membrane"], tube["fiber"], 25.0, 50)
    return Substrate("mesh", mesh, 25.0, tube)


def cyl_substrate(n, seed):
    """n z-cylinders, Gamma radii (mean 1 um), packed to 0.5 area fraction."""
    cell = 20.0 * math.sqrt(n / 64.0)
    xy, r = S.packed_cylinders(n=n, cell=cell, fraction=0.5, seed=seed)
    ss = cell / 2.0
    fp, rmax = S.cylinders_normalised(xy, r, ss)
    c = Cylinders.from_arrays(fp, rmax)
    return Substrate("cyl", c, ss, {"xy": xy, "r": r})


def tube_compartments(tube, pos, spaceScale):
    """Compartment 3 (inside a glia-type tube) or 0, with the tube index."""
    um = np.asarray(pos, np.float32).reshape(-1, 3).astype(np.float64) * spaceScale
    n = len(um)
    comp = np.zeros(n, np.uint8)
    fib = np.full(n, 0xFFFF, np.uint32)
    if n == 0:
        return comp, fib
    # Spins binned on a 2 um xy grid; each tube tests only the spins of the
    # cells under its widest cross-section (radius <= 1.2 r0, one cell of
    # margin), with the same expressions, so lower tube indices still win.
    cs = 2.0
    lo = um[:, :2].min(0)
    ix = np.floor((um[:, 0] - lo[0]) / cs).astype(np.int64)
    iy = np.floor((um[:, 1] - lo[1]) / cs).astype(np.int64)
    nx, ny = int(ix.max()) + 1, int(iy.max()) + 1
    order = np.argsort(ix * ny + iy, kind="stable")
    starts = np.searchsorted((ix * ny + iy)[order], np.arange(nx * ny + 1))
    for i, ((cx, cy), r0) in enumerate(zip(tube["centres"], tube["radii"])):
        rmax = 1.2 * r0
        x0 = max(int(np.floor((cx - rmax - lo[0]) / cs)) - 1, 0)
        x1 = min(int(np.floor((cx + rmax - lo[0]) / cs)) + 1, nx - 1)
        y0 = max(int(np.floor((cy - rmax - lo[1]) / cs)) - 1, 0)
        y1 = min(int(np.floor((cy + rmax - lo[1]) / cs)) + 1, ny - 1)
        if x0 > x1 or y0 > y1:
            continue
        idx = np.concatenate([order[starts[a * ny + y0]:starts[a * ny + y1 + 1]] for a in range(x0, x1 + 1)])
        u = um[idx]
        rz = r0 * (1 + 0.2 * np.sin(2 * np.pi * u[:, 2] / 10.0))
        sel = (np.abs(u[:, 0] - cx) < rz) & (np.abs(u[:, 1] - cy) < rz) & (comp[idx] == 0)
        sel &= np.hypot(u[:, 0] - cx, u[:, 1] - cy) < rz * np.cos(np.pi / 32)
        comp[idx[sel]] = 3
        fib[idx[sel]] = i
    return comp, fib


def cyl_regions(geom, pos, spaceScale, inner=0.7):
    """imo (0 core, 1 myelin, 2 outside) and nearest cylinder per spin."""
    xy, r = geom["xy"], geom["r"]
    um = pos[:, :2].astype(np.float64) * spaceScale
    near = np.zeros(len(pos), np.int64)
    dn = np.zeros(len(pos))
    for a in range(0, len(pos), 16384):
        d = np.hypot(um[a:a + 16384, None, 0] - xy[None, :, 0], um[a:a + 16384, None, 1] - xy[None, :, 1])
        d /= r[None, :]
        near[a:a + 16384] = np.argmin(d, 1)
        dn[a:a + 16384] = d[np.arange(len(d)), near[a:a + 16384]]
    imo = np.where(dn < inner, 0, np.where(dn <= 1.0, 1, 2)).astype(np.uint8)
    nearest = np.where(imo < 2, near, 0xFFFFFF).astype(np.uint32)
    return imo, nearest


def job_shape(rng, subs, spins_range=(4096, 1 << 20), steps_range=(2000, 10000)):
    """The first draws of make_job: substrate, spin count (log-uniform), steps
    (uniform).  A stream can size its jobs from these without generating them."""
    sub = subs[int(rng.integers(len(subs)))]
    n = int(round(math.exp(rng.uniform(math.log(spins_range[0]), math.log(spins_range[1])))))
    steps = int(rng.integers(steps_range[0], steps_range[1] + 1))
    return sub, n, steps


def make_job(rng, subs, spins_range=(4096, 1 << 20), steps_range=(2000, 10000), dirs_range=(6, 128),
             bmax=3.0, permeable=False, seed=0):
    """One job of the batching mix: substrate, spins log-uniform, steps uniform,
    dt 5-10 us, PGSE filling the walk, directions x b-values with b <= bmax."""
    sub, n, steps = job_shape(rng, subs, spins_range, steps_range)
    dt = float(rng.uniform(0.005, 0.010))
    T = steps * dt
    delta, Delta = 0.3 * T, 0.6 * T
    ndir = int(rng.integers(dirs_range[0], dirs_range[1] + 1))
    bvals = np.array([bmax / 3, 2 * bmax / 3, bmax])
    dirs = fibonacci_dirs(ndir)
    G = np.concatenate([pgse_gmag(b, delta, Delta) * dirs for b in bvals])
    gs = grad_scaled(G, sub.spaceScale).astype(F).reshape(-1, 3)
    pos = rng.uniform(-0.99, 0.99, (n, 3)).astype(F)
    if sub.kind == "mesh":
        comp, fib = tube_compartments(sub.geom, pos, sub.spaceScale)
        sd = std_devs(2.0, 2.0, 0.2, sub.spaceScale, dt)
        T2 = [80.0, 80.0, 7.5, 80.0]
        inner = 1.0
    else:
        comp, fib = cyl_regions(sub.geom, pos, sub.spaceScale)
        ss = F(sub.spaceScale)
        sd = np.array([np.sqrt(F(2) * (F(adc) / (ss * ss)) * F(dt)) for adc in (2.0, 0.2, 2.0, 0.0)], F)
        T2 = [70.0, 8.0, 80.0, 0.0]
        inner = 0.7
    perm = float(math.exp(rng.uniform(math.log(1e-4), math.log(1e-2)))) if permeable else 0.0
    return dict(sub=sub, pos=pos.reshape(-1), comp=comp, fiber=fib, steps=steps, dt=F(dt), step_sd=sd,
                T2=np.asarray(T2, F), phase_constant=phase_constant(GAMMA, dt), seed=seed, permeability=perm,
                delta=delta, Delta=Delta, grads=gs, inner=inner, n=n)
