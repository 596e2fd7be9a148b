"""Ensemble parity of the production path (Philox draws) with the reference's
own run (its multiply-with-carry draws, through the oracle pinned to the
reference's CPU code by the golden fixtures).

The two sides draw different random numbers, so they agree only in
distribution: per gradient, the signal S = |sum m e^{i phi}| / n of the GPU
run must lie within 3 combined Monte-Carlo standard errors of the
reference's, |S_gpu - S_ref| <= 3 sqrt(SE_gpu^2 + SE_ref^2), with no additive
slack.  SE is the delta-method error of |mean z| from the spins' own
contributions (the spread of Re(z e^{-i theta}), theta the mean's phase).

The reference walks every gradient afresh (dSim3/src/diffusion.cpp:553-625,
dSim2/src/diffusion.cpp:203-262).  On the GPU each gradient is a fresh
plain walk (dsim_cyl_run / dsim_mesh_run with its own Philox key), and the
batch form gives every gradient from one walk's moments.  The oracle walks
once with the reference's draws and applies each gradient's phase update
(or2_integrate_multi / or3_integrate_multi, tested against one oracle run
per gradient in tests/test_cpu_oracle.py); the walk itself does not depend
on the gradient.  Signals: dSim2 reads spins inside +-0.8
(dSim2/src/spinSystem.cpp:944-978), dSim3 every spin
(dSim3/src/spinSystem.cpp:1452-1500).
"""
import ctypes as C
import os

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

F = np.float32
Z = 3.0


def _sig_se(mag, phase, sel=None):
    """S = |mean m e^{i phi}| and its delta-method standard error."""
    m = np.asarray(mag, np.float64)
    ph = np.asarray(phase, np.float64)
    if sel is not None:
        m, ph = m[sel], ph[sel]
    z = m * np.exp(1j * ph)
    mean = z.mean()
    S = abs(mean)
    proj = (z * np.conj(mean) / S).real if S > 0 else z.real
    se = proj.std(ddof=1) / np.sqrt(len(z)) if len(z) > 1 else 0.0
    return S, se


def _check(name, S_gpu, se_gpu, S_ref, se_ref):
    S_gpu, se_gpu, S_ref, se_ref = map(np.asarray, (S_gpu, se_gpu, S_ref, se_ref))
    # 1e-12: float64 summation rounding of rows whose spread is zero (G = 0
    # without T2 gives S = 1 on both sides), not a statistical allowance
    lim = Z * np.sqrt(se_gpu ** 2 + se_ref ** 2) + 1e-12
    dz = np.abs(S_gpu - S_ref) / np.where(lim > 1e-9, lim / Z, 1.0)
    bad = np.nonzero(np.abs(S_gpu - S_ref) > lim)[0]
    assert len(bad) == 0, "%s: gradients %s outside 3 SE: gpu %s ref %s lim %s (max z %.2f)" % (
        name, bad.tolist(), S_gpu[bad], S_ref[bad], lim[bad], dz.max())
    return float(dz.max())


def _in_box(pos3, d=0.8):
    p = np.asarray(pos3).reshape(-1, 3)
    return np.all((p > -d) & (p < d), axis=1)


# --------------------------------------------------------------------------
# C1: 64 Gamma-radius cylinders, 10,000 spins, 5,000 steps, 48 PGSE gradients
# --------------------------------------------------------------------------
def test_c1_cylinders_philox_ensemble_matches_reference_run(engine):
    from dsim_gb300 import jobs as JB
    from dsim_gb300 import substrates as SS
    from dsim_gb300.engine import Batch, Spins, cyl_params, cyl_run, grad_scaled, pgse_table, phase_constant
    sub = JB.cyl_substrate(64, 1)               # 20 x 20 um cell, spaceScale 10, 0.5 packing
    c = sub.handle
    ss = F(sub.spaceScale)
    fp, rmax = SS.cylinders_normalised(sub.geom["xy"], sub.geom["r"], sub.spaceScale)
    cc, cubes, n, maxfpc, L = O.build_grid2(fp, rmax)
    gcc, gcubes, gfp = c.grid()
    assert np.array_equal(gcc, cc) and np.array_equal(gcubes, cubes)
    N, dt, steps, delta, Delta = 10_000, 0.01, 5000, 10.0, 30.0
    rng = np.random.default_rng(1)
    pos = rng.uniform(-0.995, 0.995, (N, 3)).astype(F)
    pos4 = np.zeros((N, 4), F)
    pos4[:, :3] = pos
    near = np.zeros(N, np.uint32)
    imo = np.zeros(N, np.uint32)
    O.lib().or2_find_nearest(N, pos4.reshape(-1), fp, n, L, maxfpc, cc, cubes, 1.0, near, imo)
    assert 0.3 < (imo == 0).mean() < 0.7
    dirs = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0], [1, 0, 1], [0, 1, 1]], np.float64)
    dirs /= np.linalg.norm(dirs, axis=1)[:, None]
    G = np.concatenate([lv * dirs for lv in np.linspace(0.0, 80.0, 8)])
    gs = grad_scaled(G, sub.spaceScale).astype(F).reshape(-1, 3)
    pc = phase_constant(42576.0, dt)
    w = pgse_table(steps, dt, delta, Delta)

    # the reference's run: its MWC draws, one walk giving every gradient's phase
    P = O.Params2()
    P.intraAdcScaled = P.extraAdcScaled = P.myelinAdcScaled = F(2.0) / (ss * ss)
    P.T2fiber = P.T2myelin = P.T2outside = 1e30
    P.permeability, P.innerRadiusProportion, P.spinRadius, P.deltaTime = 0.0, 1.0, 0.005, dt
    P.numCubes, P.maxFibersPerCube, P.cubeLength = n, maxfpc, L
    seed4 = np.zeros((N, 4), np.uint32)
    seed4[:, :2] = np.random.default_rng(2).integers(1, 2 ** 32 - 1, (N, 2), dtype=np.uint64)
    par = np.zeros((N, 5), F)
    par[:, 0] = 1.0
    par[:, 2] = near.astype(F)
    par[:, 3] = imo.astype(F)
    rpos = pos4.reshape(-1).copy()
    rph = O.integrate2_multi(P, rpos, seed4.reshape(-1), par.reshape(-1), fp, cc, cubes, gs, w, pc)
    rsel = _in_box(rpos.reshape(-1, 4)[:, :3])
    ref = [_sig_se(par[:, 0], rph[:, k], rsel) for k in range(len(gs))]
    # the oracle's signal for one gradient equals getMrSignal's restatement
    par_k = par.copy()
    par_k[:, 1] = rph[:, -1]
    assert np.isclose(O.lib().or2_signal(N, rpos, par_k.reshape(-1)), ref[-1][0], rtol=1e-9)

    # GPU, plain form: one fresh Philox walk per gradient
    p = cyl_params(2.0, 2.0, 2.0, sub.spaceScale, 1e30, 1e30, 1e30, 0.0, 1.0, dt, pc)
    s = Spins(N)
    plain = []
    for k, g in enumerate(gs):
        s.set_cyl(pos, None, None, imo, near)
        cyl_run(c, s, p, grad_per_step=(w[:, None] * g[None, :]).astype(F), iterations=steps, seed=101 + k)
        gp, gm, gph, _, _ = s.get_cyl()
        sums = s.signal(0.8)
        S, se = _sig_se(gm, gph, _in_box(gp))
        assert np.isclose(np.hypot(sums[0, 0], sums[0, 1]) / sums[0, 2], S, rtol=1e-6, atol=1e-7)
        plain.append((S, se))
    assert s.status() == 0
    zp = _check("C1 plain", [a for a, _ in plain], [b for _, b in plain], [a for a, _ in ref], [b for _, b in ref])

    # GPU, batch form: one walk, every gradient from its moments
    sd = [float(np.sqrt(F(2) * (F(2.0) / (ss * ss)) * F(dt)))] * 3 + [0.0]
    b = Batch((N + 31) // 32 * 32, 1)
    sid = b.add_cyl(c)
    j = b.submit(sid, pos.reshape(-1), imo, near, steps, dt, sd, [0.0] * 4, pc, 7, waveform="pgse", delta=delta,
                 Delta=Delta, inner_radius_proportion=1.0)
    b.run()
    assert b.status() == 0
    bp, bm, bmom, _, _ = b.get(j, N)
    M = bmom[:, :3].astype(np.float64) - bmom[:, 3:].astype(np.float64)
    bph = float(pc) * (M @ gs.astype(np.float64).T)
    bsel = _in_box(bp)
    sums = b.signal(j, gs, region=0.8)
    batch = []
    for k in range(len(gs)):
        S, se = _sig_se(bm, bph[:, k], bsel)
        assert np.isclose(np.hypot(sums[k, 0, 0], sums[k, 0, 1]) / sums[k, 0, 2], S, rtol=1e-9, atol=1e-12)
        batch.append((S, se))
    b.close()
    zb = _check("C1 batch", [a for a, _ in batch], [b_ for _, b_ in batch], [a for a, _ in ref],
                [b_ for _, b_ in ref])
    print("C1 max |z|: plain %.2f, batch %.2f" % (zp, zb))


# --------------------------------------------------------------------------
# permeable beaded-tube mesh, full PGSE (delta 15, Delta 40 ms at dt 5 us)
# --------------------------------------------------------------------------
def test_permeable_mesh_philox_ensemble_matches_reference_run(engine, tmp_path):
    from dsim_gb300 import substrates as SS
    from dsim_gb300.engine import (Batch, Mesh, Spins, grad_scaled, mesh_params, mesh_run, pgse_table,
                                   phase_constant, std_devs)
    from dsim_gb300.jobs import pgse_gmag
    tube = SS.beaded_tubes(n_axons=20, verts_per_ring=32, ring_spacing=0.5, length=18.0, box=20.0, closed=True,
                           membranes="G", seed=3, allow_overlap=False, bead_period=10.0)
    path = str(tmp_path / "tubes.mesh")
    SS.write_mesh_file(path, tube)
    spaceScale, D, dt, delta, Delta = 10.0, 2.0, 0.005, 15.0, 40.0
    steps = int(round((delta + Delta) / dt))           # 11,000 steps: the whole PGSE
    N, perm = 16_384, 0.01
    m = Mesh.load(path, spaceScale)
    mo = O.Mesh(path, spaceScale)
    cc, tic, maxtpc = O.populate_cubes(mo.vertices, mo.trgls, 50)
    # initial state: uniform spins, compartments by the GPU's findSpinsInFibers
    rng = np.random.default_rng(4)
    s = Spins(N)
    s.set(rng.uniform(-0.95, 0.95, 3 * N).astype(F), np.ones(N, F), np.zeros(N, F), np.zeros(N, np.uint8),
          np.full(N, 0xFFFF, np.uint16))
    m.compartments(s, seed=5)
    pos0, _, _, comp0, fib0 = s.get()
    assert 0.05 < (comp0 == 3).mean() < 0.6
    sdv = std_devs(D, D, 0.1 * D, spaceScale, dt)
    T2 = np.array([80.0, 60.0, 7.5, 40.0], F)
    pc = phase_constant(42576.0, dt)
    dirs = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0], [1, 0, 1], [0, 1, 1]], np.float64)
    dirs /= np.linalg.norm(dirs, axis=1)[:, None]
    G = np.concatenate([np.zeros((1, 3))] + [pgse_gmag(b, delta, Delta) * dirs for b in (0.3, 1.0)])
    gs = grad_scaled(G, spaceScale).astype(F).reshape(-1, 3)
    w = pgse_table(steps, dt, delta, Delta)

    # the reference's run (MWC draws), one walk for every gradient
    op = O.params3(sdv, T2, perm, dt, 50, maxtpc)
    rpos, rmag, rcomp, rfib = pos0.copy(), np.ones(N, F), comp0.copy(), fib0.copy()
    seed = np.random.default_rng(6).integers(1, 2 ** 32 - 1, 2 * N, dtype=np.uint64).astype(np.uint32)
    rcnt = np.zeros(2 * N, np.uint32)
    capped, rph = O.integrate3_multi(op, rpos, seed, rmag, rcomp, rfib, mo.vertices, mo.helpers, mo.triInfo, cc,
                                     tic, gs, w, pc, counts=rcnt)
    assert capped == 0
    ref = [_sig_se(rmag, rph[:, k]) for k in range(len(gs))]
    rcnt = rcnt.reshape(-1, 2).astype(np.float64)
    assert rcnt[:, 1].sum() > 0

    # GPU plain form: a fresh Philox walk per gradient
    p = mesh_params(sdv, T2, perm, dt, pc)
    plain, comp_frac, mag_mean = [], [], []
    for k, g in enumerate(gs):
        s.set(pos0, np.ones(N, F), np.zeros(N, F), comp0, fib0)
        mesh_run(m, s, p, grad_per_step=(w[:, None] * g[None, :]).astype(F), iterations=steps, seed=301 + k,
                 count=(k == 0))
        gp, gm, gph, gc, _ = s.get()
        sums = s.signal()
        S, se = _sig_se(gm, gph)
        assert np.isclose(np.hypot(sums[0, 0], sums[0, 1]) / sums[0, 2], S, rtol=1e-6, atol=1e-7)
        plain.append((S, se))
        comp_frac.append((gc == 3).mean())
        mag_mean.append((gm.astype(np.float64).mean(), gm.astype(np.float64).std(ddof=1) / np.sqrt(N)))
        if k == 0:
            gcnt = s.counts().astype(np.float64)
    assert s.status() == 0
    zp = _check("mesh plain", [a for a, _ in plain], [b for _, b in plain], [a for a, _ in ref],
                [b for _, b in ref])
    # compartment occupancy and magnitude (T2 by compartment) after the walk
    fr = (rcomp == 3).mean()
    se_f = np.sqrt(fr * (1 - fr) / N)
    assert abs(comp_frac[0] - fr) <= Z * np.sqrt(2) * se_f, (comp_frac[0], fr)
    rm, rse = rmag.astype(np.float64).mean(), rmag.astype(np.float64).std(ddof=1) / np.sqrt(N)
    assert abs(mag_mean[0][0] - rm) <= Z * np.hypot(mag_mean[0][1], rse), (mag_mean[0], rm)
    # reflections and permeations per spin over the walk (means of two independent walks)
    for col in (0, 1):
        a, r = gcnt[:, col], rcnt[:, col]
        lim = Z * np.hypot(a.std(ddof=1), r.std(ddof=1)) / np.sqrt(N)
        assert abs(a.mean() - r.mean()) <= lim, (col, a.mean(), r.mean(), lim)

    # GPU batch form: one walk, moments
    b = Batch((N + 31) // 32 * 32, 1)
    sid = b.add_mesh(m)
    j = b.submit(sid, pos0, comp0, fib0.astype(np.uint32), steps, dt, sdv, T2, pc, 11, permeability=perm,
                 waveform="pgse", delta=delta, Delta=Delta)
    b.run()
    assert b.status() == 0
    bp, bm, bmom, bc, _ = b.get(j, N)
    M = bmom[:, :3].astype(np.float64) - bmom[:, 3:].astype(np.float64)
    bph = float(pc) * (M @ gs.astype(np.float64).T)
    sums = b.signal(j, gs)
    batch = []
    for k in range(len(gs)):
        S, se = _sig_se(bm, bph[:, k])
        assert np.isclose(np.hypot(sums[k, 0, 0], sums[k, 0, 1]) / sums[k, 0, 2], S, rtol=1e-9, atol=1e-12)
        batch.append((S, se))
    b.close()
    zb = _check("mesh batch", [a for a, _ in batch], [b_ for _, b_ in batch], [a for a, _ in ref],
                [b_ for _, b_ in ref])
    print("mesh max |z|: plain %.2f, batch %.2f" % (zp, zb))
