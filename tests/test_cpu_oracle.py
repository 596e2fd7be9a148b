"""The CPU oracle against the reference: published Philox known answers, the
golden fixtures produced by the reference's own CPU code (tests/golden/,
generator make_golden.py) and the hand collision case of the reference's
MATLAB tests."""
import ctypes as C
import json
import os
import platform

import numpy as np
import pytest

import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_philox_known_answers():
    # Random123 known-answer vectors for philox4x32-10 (Salmon et al., SC'11)
    kat = [([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
           ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
           ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
            [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1])]
    for ctr, key, out in kat:
        assert list(O.philox(ctr, key)) == out


def _load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.mark.parametrize("name", ["mesh_am", "mesh_g"])
def test_golden_mesh(tmp_path, name):
    g = _load(name)
    prm = json.loads(str(g["params"]))
    path = tmp_path / "mesh.txt"
    path.write_bytes(g["mesh_text"].tobytes())
    m = O.Mesh(str(path), prm["spaceScale"])
    # initFibers: counts, vertices, triangles, membrane table, helpers
    assert np.array_equal(m.counts, g["counts"])
    assert np.array_equal(_bits(m.vertices), _bits(g["vertices"]))
    assert np.array_equal(m.trgls, g["trgls"])
    assert np.array_equal(m.triInfo, g["triInfo"])
    assert np.array_equal(_bits(m.helpers), _bits(g["helpers"]))
    assert np.array_equal(_bits(m.maxabs), _bits(g["maxabs"]))
    # populateCubes: per-cell lists in the reference's order
    cc, tic, maxtpc = O.populate_cubes(m.vertices, m.trgls, 50)
    assert maxtpc == int(g["grid"][2])
    assert np.array_equal(cc, g["cubeCounter"])
    dense = tic.reshape(-1, maxtpc)
    lists = np.concatenate([dense[c, :cc[c]] for c in np.nonzero(cc)[0]])
    assert np.array_equal(lists, g["cellLists"])
    # SpinSystem ctor: per-compartment sigma and T2
    from dsim_gb300.engine import std_devs
    sd = std_devs(prm["extraAdc"], prm["intraAdc"], prm["myelinAdc"], prm["spaceScale"], prm["dt"])
    assert np.array_equal(_bits(sd), _bits(g["stdDevs"]))
    # updateSpins(dt, iters) on the CPU path, replaying the reference's draws
    N, iters = prm["N"], prm["iters"]
    mag, ph, comp, fib = O.spin_fields(g["spins0"])
    pos = g["pos0"].copy()
    seed = g["seed0"].copy()
    p = O.params3(g["stdDevs"], g["T2"], prm["perm"], prm["dt"], 50, maxtpc)
    from dsim_gb300.engine import grad_scaled, phase_constant
    gs = grad_scaled([prm["gx"], prm["gy"], prm["gz"]], prm["spaceScale"])
    pc = phase_constant(prm["gamma"], prm["dt"])
    cnt = np.zeros(2 * N, np.uint32)
    capped, _ = O.integrate3(p, pos, seed, mag, ph, comp, fib, m.vertices, m.helpers, m.triInfo,
                             cc, tic, gs, pc, iters, draws=g["draws"], counts=cnt)
    assert capped == 0
    mag1, ph1, comp1, fib1 = O.spin_fields(g["spins1"])
    assert np.array_equal(_bits(pos), _bits(g["pos1"]))
    assert np.array_equal(_bits(mag), _bits(mag1))
    assert np.array_equal(_bits(ph), _bits(ph1))
    assert np.array_equal(comp, comp1)
    assert np.array_equal(fib, fib1)
    cnt = cnt.reshape(-1, 2)
    assert cnt[:, 0].sum() > 0 and cnt[:, 1].sum() > 0
    # getMrSignal(double[])
    assert np.allclose(O.signal3(mag, ph, comp), g["signal"], rtol=1e-12, atol=0)


@pytest.mark.skipif(platform.machine() != "x86_64",
                    reason="the stored draws came from the x86-64 C library's logf/cosf/sinf")
@pytest.mark.parametrize("name", ["mesh_am", "mesh_g"])
def test_golden_mwc_draws_regenerate(name):
    g = _load(name)
    prm = json.loads(str(g["params"]))
    N, iters = prm["N"], prm["iters"]
    sub = min(N, 50)
    seeds = g["seed0"].reshape(-1, 2)[:sub].copy()
    for it in range(iters):
        for i in range(sub):
            out, s = O.myrandn(seeds[i])
            seeds[i] = s
            assert np.array_equal(_bits(out), _bits(g["draws"][it, i]))


def test_golden_cylinders(tmp_path):
    g = _load("cyl")
    prm = json.loads(str(g["params"]))
    path = tmp_path / "cyl.fibers"
    path.write_bytes(g["fibers_text"].tobytes())
    fp, maxR = O.load_fibers2(str(path), prm["spaceScale"])
    assert np.array_equal(_bits(fp), _bits(g["fiberPos"]))
    assert np.float32(maxR) == g["maxR"][0]
    cc, cubes, n, maxfpc, L = O.build_grid2(fp, maxR)
    assert [n, n ** 3, maxfpc] == list(g["grid"])
    assert np.array_equal(cc, g["cubeCounter"])
    assert np.array_equal(cubes, g["cubes"])
    N, iters = prm["N"], prm["iters"]
    # findNearestFiber (assignSeeds) from the initial positions
    near = np.zeros(N, np.uint32)
    imo = np.zeros(N, np.uint32)
    O.lib().or2_find_nearest(N, g["pos0"], fp, n, L, maxfpc, cc, cubes, prm["inner"], near, imo)
    par0 = g["params0"].reshape(-1, 5)
    assert np.array_equal(near.astype(np.float32), par0[:, 2])
    assert np.array_equal(imo.astype(np.float32), par0[:, 3])
    p = O.Params2()
    ss = np.float32(prm["spaceScale"])
    p.intraAdcScaled = np.float32(prm["intraAdc"]) / (ss * ss)
    p.extraAdcScaled = np.float32(prm["extraAdc"]) / (ss * ss)
    p.myelinAdcScaled = np.float32(prm["myelinAdc"]) / (ss * ss)
    p.T2fiber, p.T2myelin, p.T2outside = prm["intraT2"], prm["myelinT2"], prm["extraT2"]
    p.permeability = prm["perm"]
    p.innerRadiusProportion = prm["inner"]
    p.spinRadius = 0.005
    p.deltaTime = prm["dt"]
    p.numCubes, p.maxFibersPerCube, p.cubeLength = n, maxfpc, L
    pos4 = g["pos0"].copy()
    seed4 = g["seed0"].copy()
    par = g["params0"].copy()
    from dsim_gb300.engine import grad_scaled, phase_constant
    gs = grad_scaled([prm["gx"], prm["gy"], prm["gz"]], prm["spaceScale"])
    pc = phase_constant(prm["gamma"], prm["dt"])
    cnt = np.zeros(2 * N, np.uint32)
    O.lib().or2_integrate(C.byref(p), N, pos4, seed4, par, fp, cc, cubes, float(gs[0]), float(gs[1]),
                          float(gs[2]), float(pc), iters, np.ascontiguousarray(g["draws"].reshape(-1)),
                          None, cnt)
    assert np.array_equal(_bits(pos4), _bits(g["pos1"]))
    assert np.array_equal(_bits(par), _bits(g["params1"]))
    assert np.array_equal(seed4.reshape(-1, 4)[:, 3], g["seed1"].reshape(-1, 4)[:, 3])
    assert cnt.reshape(-1, 2)[:, 0].sum() > 0
    assert np.isclose(O.lib().or2_signal(N, pos4, par), g["signal"][0], rtol=1e-12)


def test_matlab_hand_collision_case(tmp_path):
    """collisions01.m: one segment against one triangle; the reference reported
    the intersection point intP (6 significant digits).  One replayed step with
    sigma 1 moves the spin from oPos towards pos; the mirror image of pos
    about the triangle plane through intP must be where the spin ends."""
    c = json.load(open(os.path.join(GOLDEN, "matlab_collisions.json")))
    V = np.array([[c["x1"], c["y1"], c["z1"]], [c["x2"], c["y2"], c["z2"]],
                  [c["x3"], c["y3"], c["z3"]]], np.float32)
    path = tmp_path / "tri.mesh"
    with open(path, "w") as f:
        f.write("V\n")
        np.savetxt(f, V, fmt="%.9g")
        f.write("T\n0 1 2\nG0\n0\n")
    m = O.Mesh(str(path), 1.0)
    cc, tic, maxtpc = O.populate_cubes(m.vertices, m.trgls, 50)
    o = np.array([c["oPosx"], c["oPosy"], c["oPosz"]], np.float32)
    q = np.array([c["posx"], c["posy"], c["posz"]], np.float32)
    d = np.zeros((1, 1, 4), np.float32)
    d[0, 0, :3] = q - o
    d[0, 0, 3] = 1.0
    p = O.params3([1, 1, 1, 1], [1e30] * 4, 0.0, 0.01, 50, maxtpc)
    pos = o.copy()
    cnt = np.zeros(2, np.uint32)
    O.integrate3(p, pos, np.zeros(2, np.uint32), np.ones(1, np.float32), np.zeros(1, np.float32),
                 np.zeros(1, np.uint8), np.zeros(1, np.uint16), m.vertices, m.helpers, m.triInfo,
                 cc, tic, (0, 0, 0), 0.0, 1, draws=d, counts=cnt)
    assert list(cnt) == [1, 0]
    n = m.helpers[:3].astype(np.float64)
    ip = np.array([c["intPx"], c["intPy"], c["intPz"]])
    qq = (o.astype(np.float64) + d[0, 0, :3])
    expect = ip + (np.eye(3) - 2 * np.outer(n, n)) @ (qq - ip)
    assert np.allclose(pos, expect, atol=2e-6)


def test_fp64_oracle_moments_equal_its_phase_and_track_fp32(tmp_path):
    """The FP64 precision oracle: its moment form reproduces its own phase form
    (phase = pc * (g . M)), and its trajectories stay with the FP32 oracle's
    (pinned to the reference above) for nearly every spin."""
    from dsim_gb300.engine import grad_scaled, phase_constant, pgse_table
    g = _load("mesh_am")
    prm = json.loads(str(g["params"]))
    path = tmp_path / "mesh.txt"
    path.write_bytes(g["mesh_text"].tobytes())
    m = O.Mesh(str(path), prm["spaceScale"])
    cc, tic, maxtpc = O.populate_cubes(m.vertices, m.trgls, 50)
    N, iters = prm["N"], prm["iters"]
    p = O.params3(g["stdDevs"], g["T2"], prm["perm"], prm["dt"], 50, maxtpc)
    gs = grad_scaled([prm["gx"], prm["gy"], prm["gz"]], prm["spaceScale"]).astype(np.float64)
    pc = float(phase_constant(prm["gamma"], prm["dt"]))
    w = pgse_table(iters, prm["dt"], 0.2 * iters * prm["dt"], 0.5 * iters * prm["dt"]).astype(np.float64)
    mag0, ph0, comp0, fib0 = O.spin_fields(g["spins0"])
    v64 = m.vertices.astype(np.float64)

    def fresh():
        return (g["pos0"].astype(np.float64), mag0.astype(np.float64), comp0.copy(), fib0.copy())

    pos_a, mag_a, comp_a, fib_a = fresh()
    ph_a = np.zeros(N, np.float64)
    L = O.lib()
    L.or3_integrate_f64(C.byref(p), N, pos_a, mag_a, ph_a, comp_a, fib_a, len(m.trgls) // 3, v64, m.trgls,
                        m.triInfo, cc, tic, np.ascontiguousarray(w[:, None] * gs[None, :]).reshape(-1), pc, iters,
                        np.ascontiguousarray(g["draws"], np.float32).reshape(-1), None)
    pos_b, mag_b, comp_b, fib_b = fresh()
    capped, M = O.integrate3_f64_moments(p, pos_b, mag_b, comp_b, fib_b, v64, m.trgls, m.triInfo, cc, tic,
                                         w[None, :], g["draws"], nthreads=2)
    assert capped == 0
    assert np.array_equal(pos_a, pos_b) and np.array_equal(comp_a, comp_b)
    assert np.allclose(pc * (M[:, 0, :] @ gs), ph_a, rtol=1e-12, atol=1e-12)
    # against the FP32 oracle's (= the reference's) end positions
    d = np.abs(pos_b.reshape(-1, 3) - g["pos1"].reshape(-1, 3).astype(np.float64)).max(1)
    assert (d < 1e-5).mean() >= 0.95


def _pgse_segments(iters, nd, nD):
    """(wave value, steps) runs of a PGSE waveform as the reference's
    sequencer passes it: +G for nd steps, 0 until nD, -G for nd, 0 after."""
    w = np.zeros(iters, np.float32)
    w[:nd] = 1
    w[nD:nD + nd] = -1
    segs, k = [], 0
    while k < iters:
        j = k
        while j < iters and w[j] == w[k]:
            j += 1
        segs.append((float(w[k]), j - k))
        k = j
    return w, segs


def test_multi_gradient_walk_equals_one_run_per_gradient_mesh(tmp_path):
    """or3_integrate_multi (one walk, the phase of every gradient run) against
    or3_integrate run once per gradient over the PGSE segments with the
    reference's MWC draws: positions, magnitudes, compartments and every
    phase bit for bit."""
    from dsim_gb300.engine import grad_scaled, phase_constant
    g = _load("mesh_am")
    prm = json.loads(str(g["params"]))
    path = tmp_path / "mesh.txt"
    path.write_bytes(g["mesh_text"].tobytes())
    m = O.Mesh(str(path), prm["spaceScale"])
    cc, tic, maxtpc = O.populate_cubes(m.vertices, m.trgls, 50)
    N, iters = prm["N"], 60
    p = O.params3(g["stdDevs"], g["T2"], 0.05, prm["dt"], 50, maxtpc)
    grads = grad_scaled([[40.0, -20.0, 60.0], [0.0, 0.0, 80.0], [-70.0, 10.0, 0.0]], prm["spaceScale"])
    pc = phase_constant(prm["gamma"], prm["dt"])
    w, segs = _pgse_segments(iters, 15, 35)
    mag0, _, comp0, fib0 = O.spin_fields(g["spins0"])
    seed0 = np.random.default_rng(3).integers(1, 2 ** 32 - 1, 2 * N, dtype=np.uint64).astype(np.uint32)
    pos_m, seed_m, mag_m, comp_m, fib_m = g["pos0"].copy(), seed0.copy(), mag0.copy(), comp0.copy(), fib0.copy()
    cnt_m = np.zeros(2 * N, np.uint32)
    _, ph_m = O.integrate3_multi(p, pos_m, seed_m, mag_m, comp_m, fib_m, m.vertices, m.helpers, m.triInfo, cc, tic,
                                 grads, w, pc, counts=cnt_m, nthreads=3)
    assert cnt_m.sum() > 0
    for k in range(len(grads)):
        pos, seed, mag, comp, fib = g["pos0"].copy(), seed0.copy(), mag0.copy(), comp0.copy(), fib0.copy()
        ph = np.zeros(N, np.float32)
        for wv, n in segs:
            gk = (np.float32(wv) * grads[k]).astype(np.float32)
            O.integrate3(p, pos, seed, mag, ph, comp, fib, m.vertices, m.helpers, m.triInfo, cc, tic, gk, pc, n)
        assert np.array_equal(_bits(ph), _bits(ph_m[:, k])), k
        assert np.array_equal(_bits(pos), _bits(pos_m)) and np.array_equal(seed, seed_m)
        assert np.array_equal(_bits(mag), _bits(mag_m)) and np.array_equal(comp, comp_m)
        assert np.array_equal(fib, fib_m)


def test_multi_gradient_walk_equals_one_run_per_gradient_cylinders(tmp_path):
    """or2_integrate_multi against or2_integrate once per gradient (MWC draws)."""
    from dsim_gb300.engine import grad_scaled, phase_constant
    g = _load("cyl")
    prm = json.loads(str(g["params"]))
    path = tmp_path / "cyl.fibers"
    path.write_bytes(g["fibers_text"].tobytes())
    fp, maxR = O.load_fibers2(str(path), prm["spaceScale"])
    cc, cubes, n, maxfpc, L = O.build_grid2(fp, maxR)
    N, iters = prm["N"], 50
    p = O.Params2()
    ss = np.float32(prm["spaceScale"])
    p.intraAdcScaled = np.float32(prm["intraAdc"]) / (ss * ss)
    p.extraAdcScaled = np.float32(prm["extraAdc"]) / (ss * ss)
    p.myelinAdcScaled = np.float32(prm["myelinAdc"]) / (ss * ss)
    p.T2fiber, p.T2myelin, p.T2outside = prm["intraT2"], prm["myelinT2"], prm["extraT2"]
    p.permeability, p.innerRadiusProportion, p.spinRadius, p.deltaTime = 0.05, prm["inner"], 0.005, prm["dt"]
    p.numCubes, p.maxFibersPerCube, p.cubeLength = n, maxfpc, L
    grads = grad_scaled([[80.0, 0.0, 0.0], [0.0, 56.0, 56.0]], prm["spaceScale"])
    pc = phase_constant(prm["gamma"], prm["dt"])
    w, segs = _pgse_segments(iters, 12, 30)
    seed0 = g["seed0"].copy()
    seed0.reshape(-1, 4)[:, :2] = np.random.default_rng(4).integers(1, 2 ** 32 - 1, (N, 2), dtype=np.uint64)
    pos_m, seed_m, par_m = g["pos0"].copy(), seed0.copy(), g["params0"].copy()
    ph_m = O.integrate2_multi(p, pos_m, seed_m, par_m, fp, cc, cubes, grads, w, pc, nthreads=3)
    for k in range(len(grads)):
        pos, seed, par = g["pos0"].copy(), seed0.copy(), g["params0"].copy()
        for wv, nst in segs:
            gk = (np.float32(wv) * grads[k]).astype(np.float32)
            O.lib().or2_integrate(C.byref(p), N, pos, seed, par, fp, cc, cubes, float(gk[0]), float(gk[1]),
                                  float(gk[2]), float(pc), nst, None, None, None)
        assert not g["params0"].reshape(-1, 5)[:, 1].any()  # runs start at phase 0
        assert np.array_equal(_bits(par.reshape(-1, 5)[:, 1]), _bits(ph_m[:, k])), k
        assert np.array_equal(_bits(pos), _bits(pos_m)) and np.array_equal(seed, seed_m)
        assert np.array_equal(_bits(par.reshape(-1, 5)[:, [0, 2, 3]]), _bits(par_m.reshape(-1, 5)[:, [0, 2, 3]]))


def test_fp64_cylinder_oracle_tracks_the_fp32_oracle():
    """The FP64 cylinder walk on the reference's own draws (golden cyl
    fixture, permeable, myelin shell) stays with the FP32 oracle (pinned to
    the reference above): regions and positions agree for nearly every spin
    and the signal to float precision."""
    from dsim_gb300.engine import grad_scaled, phase_constant
    g = _load("cyl")
    prm = json.loads(str(g["params"]))
    fp = g["fiberPos"]
    cc, cubes, n, maxfpc, L = O.build_grid2(fp, float(g["maxR"][0]))
    N, iters = prm["N"], prm["iters"]
    p = O.Params2()
    ss = np.float32(prm["spaceScale"])
    p.intraAdcScaled = np.float32(prm["intraAdc"]) / (ss * ss)
    p.extraAdcScaled = np.float32(prm["extraAdc"]) / (ss * ss)
    p.myelinAdcScaled = np.float32(prm["myelinAdc"]) / (ss * ss)
    p.T2fiber, p.T2myelin, p.T2outside = prm["intraT2"], prm["myelinT2"], prm["extraT2"]
    p.permeability, p.innerRadiusProportion, p.spinRadius, p.deltaTime = prm["perm"], prm["inner"], 0.005, prm["dt"]
    p.numCubes, p.maxFibersPerCube, p.cubeLength = n, maxfpc, L
    gs = grad_scaled([prm["gx"], prm["gy"], prm["gz"]], prm["spaceScale"])
    pc = phase_constant(prm["gamma"], prm["dt"])
    par0 = g["params0"].reshape(-1, 5)
    pos3 = g["pos0"].reshape(-1, 4)[:, :3].astype(np.float64).reshape(-1).copy()
    mag = par0[:, 0].astype(np.float64).copy()
    imo = par0[:, 3].astype(np.uint32).copy()
    near = par0[:, 2].astype(np.uint32).copy()
    ph = O.integrate2_f64_multi(p, pos3, mag, imo, near, fp, cc, cubes, gs[None, :].astype(np.float64),
                                np.ones(iters), float(pc), g["draws"], nthreads=2)
    par1 = g["params1"].reshape(-1, 5)
    d = np.abs(pos3.reshape(-1, 3) - g["pos1"].reshape(-1, 4)[:, :3].astype(np.float64)).max(1)
    assert (d < 1e-5).mean() >= 0.95
    assert (imo == par1[:, 3].astype(np.uint32)).mean() >= 0.95
    ok = d < 1e-5
    assert np.allclose(ph[ok, 0], par1[ok, 1], rtol=1e-4, atol=1e-4)
    assert np.allclose(mag[ok], par1[ok, 0], rtol=1e-5)
