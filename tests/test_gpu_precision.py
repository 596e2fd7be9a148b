"""The precision form against the FP64 oracle on the same seed.

The batch's precision form (Kahan-compensated gradient moments, FP64
re-test of near-degenerate intersections, FP64 signal reduction) is run on
the GPU; the FP64 oracle (the reference's algorithm in double, recording
the same moments) walks the same spins with the same draws.  The per-
gradient signal difference must stay within 1e-3 for PGSE and OGSE
waveforms up to b = 10 ms/um^2."""
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


def test_precision_form_matches_fp64_oracle(engine, tmp_path):
    from dsim_gb300.engine import Batch, Mesh, rng_draws
    from dsim_gb300.jobs import fibonacci_dirs, pgse_gmag
    case = MeshCase(tmp_path, membranes="AM", permeability=0.05, N=512, dt=0.002)
    steps, seed = 1500, 2024
    waves, delta, Delta = _waves(steps, case.dt)
    m = Mesh.load(case.path, case.spaceScale)
    b = Batch(1 << 14, 8)
    sid = b.add_mesh(m)
    common = dict(pos=case.pos, comp=case.comp, fiber=case.fiber.astype(np.uint32), steps=steps, dt=case.dt,
                  step_sd=case.stdDevs, T2=case.T2, phase_constant=case.pc, seed=seed,
                  permeability=case.permeability, waveform="table")
    jobs = [b.submit(sid, table=w, precise=True, **common) for w in waves]
    plain = b.submit(sid, table=waves[0], precise=False, **common)
    b.run()
    assert b.status() == 0

    # FP64 oracle: same spins, same draws, same waveforms
    d = np.stack([rng_draws(seed, 0, s, case.N) for s in range(steps)])
    mo = O.Mesh(case.path, case.spaceScale)
    cc, tic, maxtpc = O.populate_cubes(mo.vertices, mo.trgls, 50)
    p = O.params3(case.stdDevs, case.T2, case.permeability, case.dt, 50, maxtpc)
    pos = case.pos.astype(np.float64)
    mag = case.mag.astype(np.float64)
    comp, fib = case.comp.copy(), case.fiber.copy()
    capped, M64 = O.integrate3_f64_moments(p, pos, mag, comp, fib, mo.vertices, mo.trgls, mo.triInfo, cc, tic,
                                           waves.astype(np.float64), d, nthreads=4)
    assert capped == 0

    dirs = fibonacci_dirs(16)
    worst = 0.0
    for k, j in enumerate(jobs):
        bpos, bmag, mom, bcomp, _ = b.get(j, case.N)
        M32 = mom[:, :3].astype(np.float64) - mom[:, 3:].astype(np.float64)
        for bval in (1.0, 3.0, 10.0):
            G = pgse_gmag(bval, delta, Delta) * dirs
            from dsim_gb300.engine import grad_scaled
            gs = grad_scaled(G, case.spaceScale).astype(np.float64)
            ph32 = float(case.pc) * (M32 @ gs.T)
            ph64 = float(case.pc) * (M64[:, k, :] @ gs.T)
            S32 = np.abs(np.sum(bmag[:, None] * np.exp(1j * ph32), 0)) / case.N
            S64 = np.abs(np.sum(mag[:, None] * np.exp(1j * ph64), 0)) / case.N
            worst = max(worst, float(np.abs(S32 - S64).max()))
            # the device's FP64 reduction of the same moments agrees with numpy
            sig = b.signal(j, gs.astype(F))
            Sd = np.hypot(sig[:, 0, 0], sig[:, 0, 1]) / sig[:, 0, 2]
            gs32 = gs.astype(F).astype(np.float64)
            S32b = np.abs(np.sum(bmag[:, None] * np.exp(1j * float(case.pc) * (M32 @ gs32.T)), 0)) / case.N
            assert np.allclose(Sd, S32b, rtol=1e-9, atol=1e-12)
        if k == 0:
            # FP32 trajectories follow the FP64 ones for nearly every spin
            dpos = np.abs(bpos.reshape(-1, 3).astype(np.float64) - pos.reshape(-1, 3)).max(1)
            assert (dpos < 1e-4).mean() >= 0.97
    assert worst <= 1e-3, worst
    tests, retests = b.precision_counts(jobs[0])
    assert tests > 0 and 0 <= retests <= tests
    assert b.precision_counts(plain) == (0, 0)
