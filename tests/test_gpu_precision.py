"""The precision form (DSIM_JOB_PRECISE) against the FP64 oracle.

The precision form evaluates the reference's mesh step in FP64 (positions,
sub-segments, triangle tests on FP64 helpers, reflections, clamp, T2 decay,
moments); the FP64 oracle is the same algorithm in double on the CPU
(oracle/dsim3_step.inc instantiated with REAL = double).  On the same spins
and draws:

* positions and magnitudes agree bit for bit, compartments, fibers and
  collision counts exactly;
* the gradient moments within 1e-12 relative (FP64 sums stored as a float
  pair between chunks);
* per-gradient signals within 1e-9 for PGSE and OGSE waveforms up to
  b = 10 ms/um^2 (the metric's bar is 1e-3);
* plain jobs in the same batch are unaffected (equal to the job alone).
"""
import numpy as np
import pytest

import oracle as O
from scenarios import MeshCase

pytestmark = pytest.mark.gpu
F = np.float32


def _waves(steps, dt):
    from dsim_gb300.engine import pgse_table
    T = steps * float(dt)
    delta, Delta = 0.35 * T, 0.6 * T
    w = [pgse_table(steps, float(dt), delta, Delta)]
    nd, nD = int(round(delta / dt)), int(round(Delta / dt))
    t = np.arange(steps) * float(dt)
    for f in (50.0, 200.0):
        x = np.zeros(steps)
        x[:nd] = np.cos(2 * np.pi * f * 1e-3 * t[:nd])
        x[nD:nD + nd] = -np.cos(2 * np.pi * f * 1e-3 * (t[nD:nD + nd] - t[nD]))
        w.append(x.astype(F))
    return np.array(w, F), delta, Delta


def _oracle(case, steps, seed, waves):
    from dsim_gb300.engine import rng_draws
    d = np.stack([rng_draws(seed, 0, s, case.N) for s in range(steps)])
    mo = O.Mesh(case.path, case.spaceScale)
    cc, tic, maxtpc = O.populate_cubes(mo.vertices, mo.trgls, 50)
    p = O.params3(case.stdDevs, case.T2, case.permeability, case.dt, 50, maxtpc)
    pos = case.pos.astype(np.float64)
    mag = case.mag.astype(np.float64)
    comp, fib = case.comp.copy(), case.fiber.copy()
    cnt = np.zeros(2 * case.N, np.uint32)
    capped, M64 = O.integrate3_f64_moments(p, pos, mag, comp, fib, mo.vertices, mo.trgls, mo.triInfo, cc, tic,
                                           np.asarray(waves, np.float64), d, counts=cnt, nthreads=4)
    assert capped == 0
    return pos.reshape(-1, 3), mag, comp, fib, cnt.reshape(-1, 2).sum(0), M64


@pytest.mark.parametrize("membranes,perm,records", [("AM", 0.05, 32), ("G", 0.3, 64), ("AM", 0.0, 32)])
def test_precision_form_walk_equals_fp64_oracle(engine, tmp_path, membranes, perm, records):
    from dsim_gb300.engine import Batch, Mesh
    case = MeshCase(tmp_path, membranes=membranes, permeability=perm, N=700, dt=0.002)
    steps, seed = 300, 91
    waves, _, _ = _waves(steps, case.dt)
    m = Mesh.load(case.path, case.spaceScale)
    m.set_records(records)
    b = Batch(1 << 14, 4)
    b.configure(chunk=7, occupancy=4, graph_chunks=2)
    sid = b.add_mesh(m)
    j = b.submit(sid, pos=case.pos, comp=case.comp, fiber=case.fiber.astype(np.uint32), steps=steps, dt=case.dt,
                 step_sd=case.stdDevs, T2=case.T2, phase_constant=case.pc, seed=seed,
                 permeability=case.permeability, waveform="table", table=waves[0], precise=True)
    b.run()
    assert b.status() == 0
    pos64, mag64, comp, fib, cnt, M64 = _oracle(case, steps, seed, waves[:1])
    gpos, gmag = b.get_precise(j, case.N)
    _, fmag, mom, gcomp, gfib = b.get(j, case.N)
    assert cnt.sum() > 0
    assert np.array_equal(b.counts(j), cnt.astype(np.uint64))
    assert np.array_equal(gpos.view(np.uint64), pos64.view(np.uint64))
    assert np.array_equal(gmag.view(np.uint64), mag64.view(np.uint64))
    assert np.array_equal(gcomp, comp)
    assert np.array_equal(gfib & 0xFFFF, fib.astype(np.uint32))
    assert np.array_equal(fmag, mag64.astype(F))
    M = mom[:, :3].astype(np.float64) - mom[:, 3:].astype(np.float64)
    scale = np.abs(M64[:, 0, :]).max()
    assert np.abs(M - M64[:, 0, :]).max() <= 1e-12 * scale
    recs, exact = b.precision_counts(j)
    assert recs > 0 and 0 < exact <= recs


def test_precision_form_signal_matches_fp64_oracle(engine, tmp_path):
    from dsim_gb300.engine import Batch, Mesh, grad_scaled
    from dsim_gb300.jobs import fibonacci_dirs, pgse_gmag
    case = MeshCase(tmp_path, membranes="AM", permeability=0.05, N=512, dt=0.002)
    steps, seed = 1500, 2024
    waves, delta, Delta = _waves(steps, case.dt)
    m = Mesh.load(case.path, case.spaceScale)
    common = dict(pos=case.pos, comp=case.comp, fiber=case.fiber.astype(np.uint32), steps=steps, dt=case.dt,
                  step_sd=case.stdDevs, T2=case.T2, phase_constant=case.pc, seed=seed,
                  permeability=case.permeability, waveform="table")
    # the plain job alone, for the mixed batch below
    b0 = Batch(1 << 14, 2)
    j0 = b0.submit(b0.add_mesh(m), table=waves[0], precise=False, **common)
    b0.run()
    alone = b0.get(j0, case.N)
    b0.close()

    b = Batch(1 << 14, 8)
    sid = b.add_mesh(m)
    jobs = [b.submit(sid, table=w, precise=True, **common) for w in waves]
    plain = b.submit(sid, table=waves[0], precise=False, **common)
    b.run()
    assert b.status() == 0
    pos64, mag64, _, _, _, M64 = _oracle(case, steps, seed, waves)

    dirs = fibonacci_dirs(16)
    worst = 0.0
    for k, j in enumerate(jobs):
        gpos, gmag = b.get_precise(j, case.N)
        assert np.array_equal(gpos.view(np.uint64), pos64.view(np.uint64))
        _, bmag, mom, _, _ = b.get(j, case.N)
        M = mom[:, :3].astype(np.float64) - mom[:, 3:].astype(np.float64)
        for bval in (1.0, 3.0, 10.0):
            G = pgse_gmag(bval, delta, Delta) * dirs
            gs = grad_scaled(G, case.spaceScale).astype(F).astype(np.float64)
            S = np.abs(np.sum(gmag[:, None] * np.exp(1j * float(case.pc) * (M @ gs.T)), 0)) / case.N
            S64 = np.abs(np.sum(mag64[:, None] * np.exp(1j * float(case.pc) * (M64[:, k, :] @ gs.T)), 0)) / case.N
            worst = max(worst, float(np.abs(S - S64).max()))
            # the device's FP64 reduction of the same moments reads the FP64 magnitudes
            sig = b.signal(j, gs.astype(F))
            Sd = np.hypot(sig[:, 0, 0], sig[:, 0, 1]) / sig[:, 0, 2]
            assert np.allclose(Sd, S, rtol=1e-9, atol=1e-12)
            assert np.allclose(Sd, S64, rtol=0, atol=1e-9)
    assert worst <= 1e-9, worst
    # the plain job sharing the batch with precision-form jobs equals the job alone
    for a, w in zip(b.get(plain, case.N), alone):
        assert np.array_equal(np.asarray(a).view(np.uint8), np.asarray(w).view(np.uint8))
    assert b.precision_counts(plain) == (0, 0)
    with pytest.raises(Exception):
        b.get_precise(plain, case.N)


def _precise_job(case, steps, seed):
    return dict(pos=case.pos, comp=case.comp, fiber=case.fiber.astype(np.uint32), steps=steps, dt=case.dt,
                step_sd=case.stdDevs, T2=case.T2, phase_constant=case.pc, seed=seed,
                permeability=case.permeability, waveform="pgse", delta=0.1, Delta=0.2, precise=True)


def test_precision_form_state_survives_mix_compaction_and_autotune(engine, tmp_path):
    """The FP64 fields follow the spins through sorts, admission of later
    jobs, compaction and the autotuner's snapshot: a precision-form job's and a
    cell-local job's positions equal the job run alone, bit for bit."""
    from dsim_gb300.engine import Batch, Mesh
    am = MeshCase(tmp_path, membranes="AM", permeability=0.05, N=600, dt=0.002)
    gl = MeshCase(tmp_path, membranes="G", permeability=0.3, N=500, dt=0.002, seed=4)
    ma, mg = Mesh.load(am.path, am.spaceScale), Mesh.load(gl.path, gl.spaceScale)
    jp, jq = _precise_job(am, 60, 5), _precise_job(gl, 140, 6)
    plain = dict(_precise_job(am, 90, 7), precise=False)
    jl = dict(_precise_job(gl, 120, 8), precise=False, local=True)

    def alone(mesh, kw, n):
        b = Batch(1 << 14, 2)
        j = b.submit(b.add_mesh(mesh), **kw)
        b.run()
        out = b.get_precise(j, n), b.counts(j)
        b.close()
        return out

    want_q = alone(mg, jq, gl.N)
    want_l = alone(mg, jl, gl.N)
    b = Batch(1 << 14, 4)
    b.configure(chunk=10, occupancy=6, graph_chunks=2)
    sa, sg = b.add_mesh(ma), b.add_mesh(mg)
    ip = b.submit(sa, **jp)
    ix = b.submit(sa, **plain)
    b.advance(30)
    iq = b.submit(sg, **jq)                 # admitted while the others run
    il = b.submit(sg, **jl)
    best, _ = b.autotune(trial_steps=20)    # snapshot and restore with FP64 fields
    b.advance(40)
    assert b.job_status(ip) == (60, True)
    b.retire(ip)
    b.compact()                             # the precision-form job q moves slots
    b.run()
    assert b.status() == 0
    (pos, mag), cnt = b.get_precise(iq, gl.N), b.counts(iq)
    assert np.array_equal(pos.view(np.uint64), want_q[0][0].view(np.uint64))
    assert np.array_equal(mag.view(np.uint64), want_q[0][1].view(np.uint64))
    assert np.array_equal(cnt, want_q[1])
    assert b.job_status(ix) == (90, True)
    (pos, mag), cnt = b.get_precise(il, gl.N), b.counts(il)   # the cell-local job likewise
    assert np.array_equal(pos.view(np.uint64), want_l[0][0].view(np.uint64))
    assert np.array_equal(cnt, want_l[1])
    b.close()


def test_cell_local_form_tracks_fp64_oracle_closer_than_plain(engine, tmp_path):
    """DSIM_JOB_LOCAL (FP32 offsets from a 1/16 lattice, FP64 re-tests of
    near-degenerate intersections, Kahan moments) against the FP64 oracle,
    with the plain FP32 form beside it on the same spins and draws.  The test
    mesh caps each axon and its myelin in one plane (coincident membranes), the
    case where a local frame needs its hit points rounded from FP64.  The
    typical position error is several times smaller than the plain form's, at
    most 1 % of spins part from the FP64 path by 1e-6, collision counts agree
    within 0.1 %, and the signal is within 1e-3 up to b = 10 ms/um^2."""
    from dsim_gb300.engine import Batch, Mesh, grad_scaled
    from dsim_gb300.jobs import fibonacci_dirs, pgse_gmag
    case = MeshCase(tmp_path, membranes="AM", permeability=0.05, N=512, dt=0.002)
    steps, seed = 1500, 2024
    waves, delta, Delta = _waves(steps, case.dt)
    m = Mesh.load(case.path, case.spaceScale)
    b = Batch(1 << 14, 4)
    sid = b.add_mesh(m)
    common = dict(pos=case.pos, comp=case.comp, fiber=case.fiber.astype(np.uint32), steps=steps, dt=case.dt,
                  step_sd=case.stdDevs, T2=case.T2, phase_constant=case.pc, seed=seed,
                  permeability=case.permeability, waveform="table", table=waves[0])
    jl = b.submit(sid, local=True, **common)
    jp = b.submit(sid, **common)
    b.run()
    assert b.status() == 0
    pos64, mag64, _, _, cnt64, M64 = _oracle(case, steps, seed, waves[:1])
    lpos, lmag = b.get_precise(jl, case.N)
    ppos = b.get(jp, case.N)[0].reshape(-1, 3).astype(np.float64)
    dl = np.abs(lpos - pos64).max(1)
    dp = np.abs(ppos - pos64).max(1)
    assert np.median(dl) * 4 < np.median(dp), (np.median(dl), np.median(dp))
    assert (dl > 1e-6).mean() <= 0.01
    assert (dl > 1e-4).mean() <= (dp > 1e-4).mean()
    for j in (jl, jp):
        c = b.counts(j).astype(np.float64)
        assert np.all(np.abs(c - cnt64) <= 0.001 * cnt64 + 2), (c, cnt64)
    recs, retests = b.precision_counts(jl)
    assert recs > 0 and 0 < retests < recs
    _, _, mom, _, _ = b.get(jl, case.N)
    M = mom[:, :3].astype(np.float64) - mom[:, 3:].astype(np.float64)
    dirs = fibonacci_dirs(16)
    for bval in (1.0, 3.0, 10.0):
        gs = grad_scaled(pgse_gmag(bval, delta, Delta) * dirs, case.spaceScale).astype(F).astype(np.float64)
        S = np.abs(np.sum(lmag[:, None] * np.exp(1j * float(case.pc) * (M @ gs.T)), 0)) / case.N
        S64 = np.abs(np.sum(mag64[:, None] * np.exp(1j * float(case.pc) * (M64[:, 0, :] @ gs.T)), 0)) / case.N
        assert np.abs(S - S64).max() <= 1e-3


@pytest.mark.parametrize("perm,inner,fine", [(0.0, 1.0, -1), (0.05, 0.7, -1), (0.05, 0.7, 0), (0.02, 1.0, 4)])
def test_cylinder_precision_form_equals_fp64_oracle(engine, tmp_path, perm, inner, fine):
    """Cylinder jobs in the precision form walk the dSim2 step in FP64: on the
    kernel's own Philox draws, positions and magnitudes equal the FP64 oracle
    (oracle/oracle_dsim2.c, or2_integrate_f64_multi) bit for bit, regions and
    nearest fibers exactly, with the fine filter grid at its default size,
    off, and k = 4; signals within 1e-9."""
    from dsim_gb300.engine import Batch, Cylinders, grad_scaled, pgse_table, phase_constant, rng_draws
    from scenarios import CylCase
    case = CylCase(tmp_path, permeability=perm, inner=inner, N=1500)
    fp, maxR = O.load_fibers2(case.path, case.spaceScale)
    cc, cubes, n, maxfpc, L = O.build_grid2(fp, maxR)
    near = np.zeros(case.N, np.uint32)
    imo = np.zeros(case.N, np.uint32)
    pos4 = np.zeros((case.N, 4), F)
    pos4[:, :3] = case.pos.reshape(-1, 3)
    O.lib().or2_find_nearest(case.N, pos4.reshape(-1), fp, n, L, maxfpc, cc, cubes, float(inner), near, imo)
    c = Cylinders.load(case.path, case.spaceScale)
    if fine >= 0:
        c.set_fine(fine)
    steps, dt, seed = 300, case.dt, 4242
    ss = F(case.spaceScale)
    adc = (F(2.0) / (ss * ss), F(0.2) / (ss * ss), F(2.0) / (ss * ss))       # intra, myelin, extra
    sd = [float(np.sqrt(F(2) * a * F(dt))) for a in adc] + [0.0]
    T2 = [70.0, 8.0, 80.0, 0.0]
    pc = phase_constant(42576.0, dt)
    table = pgse_table(steps, float(dt), 0.3 * steps * float(dt), 0.6 * steps * float(dt))
    gs = grad_scaled(np.array([[80.0, 0, 0], [0, 60.0, 30.0], [0, 0, 80.0]]), case.spaceScale).astype(F)
    b = Batch(2 * 1536, 2)
    sid = b.add_cyl(c)
    kw = dict(steps=steps, dt=dt, step_sd=sd, T2=T2, phase_constant=pc, seed=seed, permeability=perm,
              waveform="table", table=table, inner_radius_proportion=inner)
    j64 = b.submit(sid, case.pos, imo.astype(np.uint8), near, precise=True, **kw)
    j32 = b.submit(sid, case.pos, imo.astype(np.uint8), near, **kw)
    b.run()
    assert b.status() == 0
    gpos, gmag = b.get_precise(j64, case.N)
    _, _, gmom, gimo, gnear = b.get(j64, case.N)
    sums = b.signal(j64, gs)
    cnt = b.counts(j64)
    # the FP64 oracle on the same draws
    d = np.stack([rng_draws(seed, 0, t, case.N) for t in range(steps)])
    P = O.Params2()
    P.intraAdcScaled, P.myelinAdcScaled, P.extraAdcScaled = adc
    P.T2fiber, P.T2myelin, P.T2outside = 70.0, 8.0, 80.0
    P.permeability, P.innerRadiusProportion, P.spinRadius, P.deltaTime = perm, inner, 0.005, float(dt)
    P.numCubes, P.maxFibersPerCube, P.cubeLength = n, maxfpc, L
    rpos = case.pos.astype(np.float64).copy()
    rmag = np.ones(case.N)
    rimo, rnear = imo.copy(), near.copy()
    rph = O.integrate2_f64_multi(P, rpos, rmag, rimo, rnear, fp, cc, cubes, gs.astype(np.float64),
                                 table.astype(np.float64), float(pc), d, nthreads=4)
    assert np.array_equal(gpos.reshape(-1).view(np.uint64), rpos.view(np.uint64))
    assert np.array_equal(gmag.view(np.uint64), rmag.view(np.uint64))
    assert np.array_equal(gimo, rimo.astype(np.uint8))
    inside = rimo < 2
    assert np.array_equal(gnear[inside], rnear[inside])
    if perm > 0 or inner < 1.0:
        assert cnt[0] > 0
    z = rmag[:, None] * np.exp(1j * rph)
    S_ref = np.abs(z.sum(0)) / case.N
    S = np.hypot(sums[:, 0, 0], sums[:, 0, 1]) / sums[:, 0, 2]
    assert np.allclose(S, S_ref, rtol=0, atol=1e-9), (S, S_ref)
    # the plain FP32 job in the same batch still equals a batch of its own
    b2 = Batch(1536, 1)
    j2 = b2.submit(b2.add_cyl(c), case.pos, imo.astype(np.uint8), near, **kw)
    b2.run()
    for a1, a2 in zip(b.get(j32, case.N), b2.get(j2, case.N)):
        assert np.array_equal(np.asarray(a1).view(np.uint8), np.asarray(a2).view(np.uint8))
    b.close()
    b2.close()


@pytest.mark.parametrize("perm,inner,fine", [(0.0, 1.0, -1), (0.05, 0.7, -1), (0.02, 0.7, 0)])
def test_cylinder_cell_local_form_tracks_fp64_oracle(engine, tmp_path, perm, inner, fine):
    """Cylinder jobs in the cell-local form (DSIM_JOB_LOCAL: FP32 offsets from a
    1/16 lattice, distances in the local frame, FP64 decisions inside the FP32
    error band, Kahan moments) against the FP64 oracle on the kernel's own
    Philox draws, with the plain FP32 form beside it: the typical position
    error is several times smaller than the plain form's, at most 1 % of spins
    part from the FP64 path by 1e-6, regions and collision counts agree within
    0.5 %, signals within 1e-4; the plain job is unchanged by the local one in
    its batch."""
    from dsim_gb300.engine import Batch, Cylinders, grad_scaled, pgse_table, phase_constant, rng_draws
    from scenarios import CylCase
    case = CylCase(tmp_path, permeability=perm, inner=inner, N=1500)
    fp, maxR = O.load_fibers2(case.path, case.spaceScale)
    cc, cubes, n, maxfpc, L = O.build_grid2(fp, maxR)
    near = np.zeros(case.N, np.uint32)
    imo = np.zeros(case.N, np.uint32)
    pos4 = np.zeros((case.N, 4), F)
    pos4[:, :3] = case.pos.reshape(-1, 3)
    O.lib().or2_find_nearest(case.N, pos4.reshape(-1), fp, n, L, maxfpc, cc, cubes, float(inner), near, imo)
    c = Cylinders.load(case.path, case.spaceScale)
    if fine >= 0:
        c.set_fine(fine)
    steps, dt, seed = 300, case.dt, 4243
    ss = F(case.spaceScale)
    adc = (F(2.0) / (ss * ss), F(0.2) / (ss * ss), F(2.0) / (ss * ss))       # intra, myelin, extra
    sd = [float(np.sqrt(F(2) * a * F(dt))) for a in adc] + [0.0]
    T2 = [70.0, 8.0, 80.0, 0.0]
    pc = phase_constant(42576.0, dt)
    table = pgse_table(steps, float(dt), 0.3 * steps * float(dt), 0.6 * steps * float(dt))
    gs = grad_scaled(np.array([[80.0, 0, 0], [0, 60.0, 30.0], [0, 0, 80.0]]), case.spaceScale).astype(F)
    b = Batch(2 * 1536, 2)
    sid = b.add_cyl(c)
    kw = dict(steps=steps, dt=dt, step_sd=sd, T2=T2, phase_constant=pc, seed=seed, permeability=perm,
              waveform="table", table=table, inner_radius_proportion=inner)
    jl = b.submit(sid, case.pos, imo.astype(np.uint8), near, local=True, **kw)
    j32 = b.submit(sid, case.pos, imo.astype(np.uint8), near, **kw)
    b.run()
    assert b.status() == 0
    lpos, lmag = b.get_precise(jl, case.N)
    _, _, _, limo, _ = b.get(jl, case.N)
    ppos = b.get(j32, case.N)[0].reshape(-1, 3).astype(np.float64)
    sums = b.signal(jl, gs)
    d = np.stack([rng_draws(seed, 0, t, case.N) for t in range(steps)])
    P = O.Params2()
    P.intraAdcScaled, P.myelinAdcScaled, P.extraAdcScaled = adc
    P.T2fiber, P.T2myelin, P.T2outside = 70.0, 8.0, 80.0
    P.permeability, P.innerRadiusProportion, P.spinRadius, P.deltaTime = perm, inner, 0.005, float(dt)
    P.numCubes, P.maxFibersPerCube, P.cubeLength = n, maxfpc, L
    rpos = case.pos.astype(np.float64).copy()
    rmag = np.ones(case.N)
    rimo, rnear = imo.copy(), near.copy()
    rph = O.integrate2_f64_multi(P, rpos, rmag, rimo, rnear, fp, cc, cubes, gs.astype(np.float64),
                                 table.astype(np.float64), float(pc), d, nthreads=4)
    rpos = rpos.reshape(-1, 3)
    dl = np.abs(lpos - rpos).max(1)
    dp = np.abs(ppos - rpos).max(1)
    assert np.median(dl) * 4 < np.median(dp), (np.median(dl), np.median(dp))
    assert (dl > 1e-6).mean() <= 0.01
    assert (limo != rimo.astype(np.uint8)).mean() <= 0.005
    if perm > 0 or inner < 1.0:
        cl, c32 = b.counts(jl).astype(np.float64), b.counts(j32).astype(np.float64)
        assert cl[0] > 0 and abs(cl[0] - c32[0]) <= 0.005 * c32[0] + 2, (cl, c32)
    tests, exact = b.precision_counts(jl)
    assert tests > 0 and exact < tests
    z = rmag[:, None] * np.exp(1j * rph)
    S_ref = np.abs(z.sum(0)) / case.N
    S = np.hypot(sums[:, 0, 0], sums[:, 0, 1]) / sums[:, 0, 2]
    assert np.abs(S - S_ref).max() <= 1e-4, (S, S_ref)
    b2 = Batch(1536, 1)
    j2 = b2.submit(b2.add_cyl(c), case.pos, imo.astype(np.uint8), near, **kw)
    b2.run()
    for a1, a2 in zip(b.get(j32, case.N), b2.get(j2, case.N)):
        assert np.array_equal(np.asarray(a1).view(np.uint8), np.asarray(a2).view(np.uint8))
    b.close()
    b2.close()
