"""The seeded job mix of the batching and serving benches (dsim_gb300/jobs.py),
on the host: every draw within its stated range, b-values at most bmax,
permeability log-uniform in [1e-4, 1e-2] when asked for, and the same seed
giving the same jobs.  Substrate handles are not needed for generation, so
the substrates here carry the geometry only."""
import math

import numpy as np

from dsim_gb300 import jobs as JB
from dsim_gb300 import substrates as S


def _subs():
    tube = S.beaded_tubes(n_axons=20, verts_per_ring=12, ring_spacing=1.0, length=50.0, box=50.0, seed=3)
    xy, r = S.packed_cylinders(n=16, cell=10.0, fraction=0.5, seed=2)
    return [JB.Substrate("mesh", None, 25.0, tube), JB.Substrate("cyl", None, 5.0, {"xy": xy, "r": r})]


def _bvalue(G, delta, Delta):
    """b (ms/um^2) of PGSE |G| (mT/m): the inverse of pgse_gmag."""
    return (2 * math.pi * JB.GAMMA * 1e-9 * G * delta) ** 2 * (Delta - delta / 3.0)


def test_job_draws_within_ranges_and_b_at_most_bmax():
    subs = _subs()
    rng = np.random.default_rng(7)
    for k in range(40):
        j = JB.make_job(rng, subs, spins_range=(4096, 65536), steps_range=(200, 400), dirs_range=(6, 20),
                        bmax=3.0, permeable=(k % 2 == 1), seed=k)
        assert 4096 <= j["n"] <= 65536 and len(j["pos"]) == 3 * j["n"]
        assert 200 <= j["steps"] <= 400
        assert 0.005 <= float(j["dt"]) <= 0.010
        assert np.all(np.abs(j["pos"]) <= 0.99)
        assert len(j["comp"]) == j["n"] and len(j["fiber"]) == j["n"]
        assert j["delta"] < j["Delta"] and j["Delta"] + j["delta"] <= j["steps"] * float(j["dt"]) + 1e-9
        ndir = len(j["grads"]) // 3
        assert 6 <= ndir <= 20 and len(j["grads"]) == 3 * ndir
        ss = j["sub"].spaceScale
        G = np.linalg.norm(j["grads"].astype(np.float64), axis=1) / (1e-9 * ss)   # mT/m
        b = _bvalue(G, j["delta"], j["Delta"])
        assert b.max() <= 3.0 * (1 + 1e-5) and b.min() >= 1.0 * (1 - 1e-5)
        if k % 2:
            assert 1e-4 <= j["permeability"] <= 1e-2
        else:
            assert j["permeability"] == 0.0
        assert j["sub"].kind in ("mesh", "cyl")
        if j["sub"].kind == "mesh":
            assert set(np.unique(j["comp"])) <= {0, 1, 2, 3}
        else:
            assert set(np.unique(j["comp"])) <= {0, 1, 2}


def test_same_seed_same_mix():
    subs = _subs()
    a = [JB.make_job(np.random.default_rng(11), subs, spins_range=(4096, 8192), steps_range=(100, 200), seed=1)
         for _ in range(2)]
    for key in ("n", "steps", "delta", "Delta", "permeability"):
        assert a[0][key] == a[1][key]
    for key in ("pos", "comp", "fiber", "grads", "step_sd", "T2"):
        assert np.array_equal(np.asarray(a[0][key]), np.asarray(a[1][key]))


def test_fibonacci_directions_are_unit_and_spread():
    for n in (6, 32, 64):
        d = JB.fibonacci_dirs(n)
        assert d.shape == (n, 3)
        assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-6)
        # no two directions coincide
        c = d @ d.T - np.eye(n) * 2
        assert c.max() < 0.999


def _tube_compartments_every_tube(tube, pos, spaceScale):
    """Every spin against every tube in index order (the first tube holding a
    spin wins): the definition the binned tube_compartments must equal."""
    um = pos.astype(np.float64) * spaceScale
    comp = np.zeros(len(pos), np.uint8)
    fib = np.full(len(pos), 0xFFFF, np.uint32)
    for i, ((cx, cy), r0) in enumerate(zip(tube["centres"], tube["radii"])):
        rz = r0 * (1 + 0.2 * np.sin(2 * np.pi * um[:, 2] / 10.0))
        sel = (np.abs(um[:, 0] - cx) < rz) & (np.abs(um[:, 1] - cy) < rz) & (comp == 0)
        sel &= np.hypot(um[:, 0] - cx, um[:, 1] - cy) < rz * np.cos(np.pi / 32)
        comp[sel] = 3
        fib[sel] = i
    return comp, fib


def test_binned_tube_compartments_equal_every_tube_scan():
    tube = S.beaded_tubes(n_axons=60, verts_per_ring=12, ring_spacing=1.0, length=50.0, box=50.0, seed=5,
                          allow_overlap=True)
    rng = np.random.default_rng(11)
    pos = rng.uniform(-0.99, 0.99, (60000, 3)).astype(np.float32)
    # spins on tube surfaces and axes too
    c = np.asarray(tube["centres"], np.float64)[:, None, :]
    r = np.asarray(tube["radii"], np.float64)[:, None]
    a = rng.uniform(0, 2 * np.pi, (len(c), 50))
    z = rng.uniform(-24.0, 24.0, (len(c), 50))
    rz = r * (1 + 0.2 * np.sin(2 * np.pi * z / 10.0))
    for k in (0.0, 0.5, np.cos(np.pi / 32), 1.0, 1.2):
        p = np.stack([c[..., 0] + k * rz * np.cos(a), c[..., 1] + k * rz * np.sin(a), z], -1).reshape(-1, 3)
        pos = np.concatenate([pos, (p / 25.0).astype(np.float32)])
    got = JB.tube_compartments(tube, pos, 25.0)
    want = _tube_compartments_every_tube(tube, pos, 25.0)
    assert (want[0] == 3).sum() > 1000
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
    e = JB.tube_compartments(tube, np.zeros((0, 3), np.float32), 25.0)
    assert len(e[0]) == 0 and len(e[1]) == 0


def test_job_shape_is_make_jobs_first_draws():
    subs = _subs()
    for k in range(20):
        sub, n, steps = JB.job_shape(np.random.default_rng([9, k]), subs, (4096, 1 << 20), (2000, 10000))
        j = JB.make_job(np.random.default_rng([9, k]), subs, spins_range=(4096, 1 << 20), steps_range=(2000, 10000),
                        permeable=True, seed=k)
        assert j["sub"] is sub and j["n"] == n and j["steps"] == steps
