"""GPU parity of the cylinder (dSim2) hot path against the CPU oracle
(the C restatement of dSim2's cpuIntegrate, pinned by the golden fixtures)."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from scenarios import CylCase, draws

pytestmark = pytest.mark.gpu


def _oracle(case, fp, cc, cubes, n, maxfpc, L, iters, d, near, imo):
    p = O.Params2()
    ss = np.float32(case.spaceScale)
    p.intraAdcScaled = np.float32(case.D) / (ss * ss)
    p.extraAdcScaled = np.float32(case.D) / (ss * ss)
    p.myelinAdcScaled = np.float32(0.1 * case.D) / (ss * ss)
    p.T2fiber, p.T2myelin, p.T2outside = 70.0, 8.0, 80.0
    p.permeability = case.permeability
    p.innerRadiusProportion = case.inner
    p.spinRadius = 0.005
    p.deltaTime = case.dt
    p.numCubes, p.maxFibersPerCube, p.cubeLength = n, maxfpc, L
    N = case.N
    pos4 = np.zeros(4 * N, np.float32)
    pos4.reshape(-1, 4)[:, :3] = case.pos.reshape(-1, 3)
    seed4 = np.zeros(4 * N, np.uint32)
    par = np.zeros(5 * N, np.float32)
    par.reshape(-1, 5)[:, 0] = 1.0
    par.reshape(-1, 5)[:, 2] = near.astype(np.float32)
    par.reshape(-1, 5)[:, 3] = imo.astype(np.float32)
    cnt = np.zeros(2 * N, np.uint32)
    O.lib().or2_integrate(C.byref(p), N, pos4, seed4, par, fp, cc, cubes, float(case.g[0]),
                          float(case.g[1]), float(case.g[2]), float(case.pc), iters,
                          np.ascontiguousarray(d.reshape(-1)), None, cnt)
    return pos4.reshape(-1, 4), par.reshape(-1, 5), cnt.reshape(-1, 2)


def _setup(case):
    fp, maxR = O.load_fibers2(case.path, case.spaceScale)
    cc, cubes, n, maxfpc, L = O.build_grid2(fp, maxR)
    near = np.zeros(case.N, np.uint32)
    imo = np.zeros(case.N, np.uint32)
    pos4 = np.zeros(4 * case.N, np.float32)
    pos4.reshape(-1, 4)[:, :3] = case.pos.reshape(-1, 3)
    O.lib().or2_find_nearest(case.N, pos4, fp, n, L, maxfpc, cc, cubes, float(case.inner), near, imo)
    return fp, maxR, cc, cubes, n, maxfpc, L, near, imo


@pytest.mark.parametrize("perm,inner", [(0.0, 1.0), (0.05, 0.7)])
def test_cyl_replay_bit_parity_native(engine, tmp_path, perm, inner):
    from dsim_gb300.engine import Cylinders, Spins, cyl_params, cyl_run
    case = CylCase(tmp_path, permeability=perm, inner=inner, N=3000)
    fp, maxR, cc, cubes, n, maxfpc, L, near, imo = _setup(case)
    c = Cylinders.load(case.path, case.spaceScale)
    gcc, gcubes, gfp = c.grid()
    assert (c.numCubes, c.maxFPC) == (n, maxfpc)
    assert np.array_equal(gfp.view(np.uint32), fp.view(np.uint32))
    assert np.array_equal(gcc, cc) and np.array_equal(gcubes, cubes)
    iters = 80
    d = draws(iters, case.N, seed=21)
    rpos, rpar, rcnt = _oracle(case, fp, cc, cubes, n, maxfpc, L, iters, d, near, imo)
    s = Spins(case.N)
    s.set_cyl(case.pos, None, None, imo, near)
    p = cyl_params(case.D, case.D, 0.1 * case.D, case.spaceScale, 70.0, 8.0, 80.0, case.permeability,
                   case.inner, case.dt, case.pc)
    cyl_run(c, s, p, g=case.g, iterations=iters, draws=d, count=True)
    pos, mag, ph, gimo, gnear = s.get_cyl()
    cnt = s.counts()
    assert s.status() == 0
    assert cnt.sum() > 0
    assert np.array_equal(cnt, rcnt)
    assert np.array_equal(pos.reshape(-1, 3).view(np.uint32), rpos[:, :3].view(np.uint32))
    assert np.array_equal(ph.view(np.uint32), rpar[:, 1].view(np.uint32))
    assert np.array_equal(mag.view(np.uint32), rpar[:, 0].view(np.uint32))
    assert np.array_equal(gimo, rpar[:, 3].astype(np.uint32))
    inside = gimo < 2
    assert np.array_equal(gnear[inside], rpar[inside, 2].astype(np.uint32))


@pytest.mark.parametrize("fine", [-1, 0, 3])
def test_cyl_replay_bit_parity_dsim2_abi(engine, tmp_path, fine):
    """Replay through the reference-facing dSim2 C-ABI (libdsim2.so), with
    the fine filter grid at its default size (-1), off (0) and k = 3."""
    from dsim_gb300 import _lib
    L2 = _lib.abi2()
    L2.dsim2_set_fine(fine)
    case = CylCase(tmp_path, permeability=0.05, inner=0.7, N=2000)
    fp, maxR, cc, cubes, n, maxfpc, L, near, imo = _setup(case)
    iters = 50
    d = draws(iters, case.N, seed=9)
    rpos, rpar, rcnt = _oracle(case, fp, cc, cubes, n, maxfpc, L, iters, d, near, imo)

    def dev(arr):
        p = C.c_void_p()
        L2.allocateArray(C.byref(p), arr.nbytes)
        L2.copyArrayToDevice(p, arr.ctypes.data, 0, arr.nbytes)
        return p

    pos4 = np.zeros((case.N, 4), np.float32)
    pos4[:, :3] = case.pos.reshape(-1, 3)
    seed4 = np.zeros((case.N, 4), np.uint32)
    seed4[:, 2] = imo + 1
    seed4[:, 3] = near
    dPos, dSeed = dev(pos4), dev(seed4)
    dFib, dCc, dCubes = dev(fp), dev(cc), dev(cubes)
    dDraws, dCnt = dev(d.reshape(-1)), dev(np.zeros(2 * case.N, np.uint32))
    L2.bindFiberList(dFib, len(fp) // 4)
    L2.bindCubeList(dCubes, len(cubes))
    L2.dsim2_set_replay(dDraws, dCnt)
    ss = np.float32(case.spaceScale)
    adc = lambda a: float(np.float32(a) / (ss * ss))
    g = _lib.Float3(*[float(x) for x in case.g])
    L2.integrateSystem(dPos, dSeed, float(case.dt), dFib, float(case.permeability), adc(case.D),
                       adc(case.D), adc(0.1 * case.D), case.N, g, float(case.pc), dCc, dCubes,
                       float(L), n, maxfpc, float(case.inner), iters)
    L2.dsim2_set_replay(None, None)
    assert L2.dsim2_last_status() == 0, L2.dsim2_last_error()
    out = np.zeros_like(pos4)
    sd = np.zeros_like(seed4)
    cnt = np.zeros(2 * case.N, np.uint32)
    L2.copyArrayFromDevice(out.ctypes.data, dPos, 0, out.nbytes)
    L2.copyArrayFromDevice(sd.ctypes.data, dSeed, 0, sd.nbytes)
    L2.copyArrayFromDevice(cnt.ctypes.data, dCnt, 0, cnt.nbytes)
    assert L2.dsim2_status() == 0
    assert np.array_equal(cnt.reshape(-1, 2), rcnt)
    assert np.array_equal(out[:, :3].view(np.uint32), rpos[:, :3].view(np.uint32))
    assert np.array_equal(out[:, 3].view(np.uint32), rpar[:, 1].view(np.uint32))
    assert np.array_equal(sd[:, 2] - 1, rpar[:, 3].astype(np.uint32))
    for p in (dPos, dSeed, dFib, dCc, dCubes, dDraws, dCnt):
        L2.freeArray(p)
    L2.dsim2_set_fine(-1)


def test_cyl_dsim2_abi_grid_rewritten_in_place(engine, tmp_path):
    """The caller overwrites the fibers and grid in the same device arrays
    between two integrateSystem calls: the second call walks the new fibers
    (the fine grid follows the contents, not the pointers), bit for bit with
    the oracle run on the same two grids."""
    from dsim_gb300 import _lib
    L2 = _lib.abi2()
    L2.dsim2_set_fine(-1)
    case = CylCase(tmp_path, permeability=0.05, inner=0.7, N=2000)
    fp, maxR, cc, cubes, n, maxfpc, L, near, imo = _setup(case)
    fp2 = fp.copy().reshape(-1, 4)
    fp2[:, 0] = np.where(fp2[:, 0] == 2.0, fp2[:, 0], fp2[:, 0] + np.float32(0.05))
    fp2[:, 1] = np.where(fp2[:, 1] == 2.0, fp2[:, 1], fp2[:, 1] - np.float32(0.03))
    fp2 = fp2.reshape(-1)
    cc2, cubes2, n2, maxfpc2, L2len = O.build_grid2(fp2, maxR)
    assert (n2, maxfpc2) == (n, maxfpc) and len(cubes2) == len(cubes)
    it1, it2 = 30, 30
    d = draws(it1 + it2, case.N, seed=12)
    # oracle: the first segment on the first grid, the second on the second
    rpos, rpar, rcnt = _oracle(case, fp, cc, cubes, n, maxfpc, L, it1, d[:it1], near, imo)
    p = O.Params2()
    ss = np.float32(case.spaceScale)
    p.intraAdcScaled = np.float32(case.D) / (ss * ss)
    p.extraAdcScaled = np.float32(case.D) / (ss * ss)
    p.myelinAdcScaled = np.float32(0.1 * case.D) / (ss * ss)
    p.T2fiber, p.T2myelin, p.T2outside = 70.0, 8.0, 80.0
    p.permeability = case.permeability
    p.innerRadiusProportion = case.inner
    p.spinRadius = 0.005
    p.deltaTime = case.dt
    p.numCubes, p.maxFibersPerCube, p.cubeLength = n, maxfpc, L2len
    pos4 = np.ascontiguousarray(rpos.reshape(-1))
    par = np.ascontiguousarray(rpar.reshape(-1))
    seed4 = np.zeros(4 * case.N, np.uint32)
    cnt = np.ascontiguousarray(rcnt.reshape(-1))
    O.lib().or2_integrate(C.byref(p), case.N, pos4, seed4, par, fp2, cc2, cubes2, float(case.g[0]),
                          float(case.g[1]), float(case.g[2]), float(case.pc), it2,
                          np.ascontiguousarray(d[it1:].reshape(-1)), None, cnt)

    def dev(arr):
        q = C.c_void_p()
        L2.allocateArray(C.byref(q), arr.nbytes)
        L2.copyArrayToDevice(q, arr.ctypes.data, 0, arr.nbytes)
        return q

    g4 = np.zeros((case.N, 4), np.float32)
    g4[:, :3] = case.pos.reshape(-1, 3)
    sd4 = np.zeros((case.N, 4), np.uint32)
    sd4[:, 2] = imo + 1
    sd4[:, 3] = near
    dPos, dSeed = dev(g4), dev(sd4)
    dFib, dCc, dCubes = dev(fp), dev(cc), dev(cubes)
    dDraws, dCnt = dev(d.reshape(-1)), dev(np.zeros(2 * case.N, np.uint32))
    L2.bindFiberList(dFib, len(fp) // 4)
    L2.bindCubeList(dCubes, len(cubes))
    ss = np.float32(case.spaceScale)
    adc = lambda a: float(np.float32(a) / (ss * ss))
    g = _lib.Float3(*[float(x) for x in case.g])
    for seg, (fib_h, cc_h, cubes_h, L_seg, its, off) in enumerate(
            [(fp, cc, cubes, L, it1, 0), (fp2, cc2, cubes2, L2len, it2, it1)]):
        if seg:
            L2.copyArrayToDevice(dFib, fib_h.ctypes.data, 0, fib_h.nbytes)
            L2.copyArrayToDevice(dCc, cc_h.ctypes.data, 0, cc_h.nbytes)
            L2.copyArrayToDevice(dCubes, cubes_h.ctypes.data, 0, cubes_h.nbytes)
        L2.dsim2_set_replay(C.c_void_p(dDraws.value + off * case.N * 16), dCnt)
        L2.integrateSystem(dPos, dSeed, float(case.dt), dFib, float(case.permeability), adc(case.D),
                           adc(case.D), adc(0.1 * case.D), case.N, g, float(case.pc), dCc, dCubes,
                           float(L_seg), n, maxfpc, float(case.inner), its)
        assert L2.dsim2_last_status() == 0, L2.dsim2_last_error()
    L2.dsim2_set_replay(None, None)
    out = np.zeros_like(g4)
    sd = np.zeros_like(sd4)
    gcnt = np.zeros(2 * case.N, np.uint32)
    L2.copyArrayFromDevice(out.ctypes.data, dPos, 0, out.nbytes)
    L2.copyArrayFromDevice(sd.ctypes.data, dSeed, 0, sd.nbytes)
    L2.copyArrayFromDevice(gcnt.ctypes.data, dCnt, 0, gcnt.nbytes)
    assert L2.dsim2_status() == 0
    assert np.array_equal(gcnt, cnt) and gcnt.sum() > 0
    assert np.array_equal(out[:, :3].view(np.uint32), pos4.reshape(-1, 4)[:, :3].view(np.uint32))
    assert np.array_equal(out[:, 3].view(np.uint32), par.reshape(-1, 5)[:, 1].view(np.uint32))
    assert np.array_equal(sd[:, 2] - 1, par.reshape(-1, 5)[:, 3].astype(np.uint32))
    for q in (dPos, dSeed, dFib, dCc, dCubes, dDraws, dCnt):
        L2.freeArray(q)


def _mixed_fibers(seed, per_axis=24):
    """Fibers along x, y and z (the axis coordinate 2.0), overlapping freely."""
    rng = np.random.default_rng(seed)
    rows = []
    for axis in (0, 1, 2):
        for _ in range(per_axis):
            c = rng.uniform(-0.9, 0.9, 3)
            r = rng.uniform(0.03, 0.12)
            c[axis] = 2.0
            rows.append([c[0], c[1], c[2], r * r])
    fp = np.array(rows, np.float32).reshape(-1)
    return fp, float(np.sqrt(fp.reshape(-1, 4)[:, 3].max()))


@pytest.mark.parametrize("perm,inner", [(0.0, 1.0), (0.05, 0.7)])
def test_cyl_fine_grid_equals_full_list_scan(engine, perm, inner):
    """The fine filter grid against the full scan of the reference grid's
    lists, bit for bit: mixed fiber axes, Philox draws, several fine sizes,
    and a third of the spins labelled outside while inside a fiber (their
    first test rejects, so the rest of the list runs at the old position)."""
    from dsim_gb300.engine import Cylinders, Spins, cyl_params, cyl_run
    fp, maxR = _mixed_fibers(5)
    cc, cubes, n, maxfpc, L = O.build_grid2(fp, maxR)
    N = 24000
    rng = np.random.default_rng(6)
    pos = rng.uniform(-0.99, 0.99, (N, 3)).astype(np.float32)
    pos4 = np.zeros((N, 4), np.float32)
    pos4[:, :3] = pos
    near = np.zeros(N, np.uint32)
    imo = np.zeros(N, np.uint32)
    O.lib().or2_find_nearest(N, pos4.reshape(-1), fp, n, L, maxfpc, cc, cubes, float(inner), near, imo)
    imo[::3] = 2
    c = Cylinders.from_arrays(fp, maxR)
    assert (c.numCubes, c.maxFPC) == (n, maxfpc)
    assert c.fine_info()["k"] >= 2 and c.fine_info()["entries"] > 0
    p = cyl_params(2.0, 2.0, 0.2, 10.0, 70.0, 8.0, 80.0, perm, inner, 0.01, 0.5)
    outs = {}
    for k in (0, 2, 7, 16, None):
        if k is None:
            c.free()
            c = Cylinders.from_arrays(fp, maxR)   # the default size again
        else:
            c.set_fine(k)
            assert c.fine_info()["k"] == k
        s = Spins(N)
        s.set_cyl(pos.reshape(-1), None, None, imo, near)
        cyl_run(c, s, p, g=(0.01, 0.02, -0.01), iterations=400, seed=17, count=True)
        assert s.status() == 0
        outs[k] = (s.get_cyl(), s.counts())
    (pos0, mag0, ph0, imo0, near0), cnt0 = outs[0]
    assert cnt0[:, 0].sum() > 0
    if perm > 0:
        assert cnt0[:, 1].sum() > 0
    for k, ((pk, mk, phk, ik, nk), ck) in outs.items():
        assert np.array_equal(pk.view(np.uint32), pos0.view(np.uint32)), k
        assert np.array_equal(phk.view(np.uint32), ph0.view(np.uint32)), k
        assert np.array_equal(mk.view(np.uint32), mag0.view(np.uint32)), k
        assert np.array_equal(ik, imo0) and np.array_equal(nk, near0) and np.array_equal(ck, cnt0), k


def test_cyl_fine_grid_in_a_batch(engine):
    """A cylinder job in a batch, with and without the fine grid: the same
    spins, moments and counts."""
    from dsim_gb300._lib import DsimError
    from dsim_gb300.engine import Batch, Cylinders
    fp, maxR = _mixed_fibers(8)
    cc, cubes, n, maxfpc, L = O.build_grid2(fp, maxR)
    N = 5000
    rng = np.random.default_rng(9)
    pos = rng.uniform(-0.99, 0.99, (N, 3)).astype(np.float32)
    pos4 = np.zeros((N, 4), np.float32)
    pos4[:, :3] = pos
    near = np.zeros(N, np.uint32)
    imo = np.zeros(N, np.uint32)
    O.lib().or2_find_nearest(N, pos4.reshape(-1), fp, n, L, maxfpc, cc, cubes, 0.7, near, imo)
    res = []
    for fine in (True, False):
        c = Cylinders.from_arrays(fp, maxR)
        if not fine:
            c.set_fine(0)
        b = Batch(N + 32, 2)
        sid = b.add_cyl(c)
        with pytest.raises(DsimError, match="in a batch"):
            c.set_fine(3)   # the batch holds the substrate's device view
        j = b.submit(sid, pos.reshape(-1), imo.astype(np.uint8), near, 300, 0.01, [0.02, 0.02, 0.01, 0.0],
                     [0.0] * 4, 0.5, 3, permeability=0.05, waveform="pgse", delta=1.0, Delta=2.0,
                     inner_radius_proportion=0.7)
        b.run()
        res.append((b.get(j, N), b.counts(j)))
        b.close()
        c.set_fine(0)   # allowed again once the batch is gone
        c.free()
    (a, ca), (b_, cb) = res
    assert ca[0] > 0 and np.array_equal(ca, cb)
    for x, y in zip(a, b_):
        assert np.array_equal(np.asarray(x).view(np.uint8), np.asarray(y).view(np.uint8))


@pytest.mark.parametrize("nfib,rmax,seed", [(64, 0.1, 1), (150, 0.1, 5), (560, 0.05, 2), (3500, 0.02, 3), (4000, 0.02, 3), (10, 0.05, 4)])
def test_cyl_grid_built_on_the_gpu_equals_add_entities(engine, nfib, rmax, seed):
    """The grid dsim_cyl_create builds on the GPU equals addEntities
    (dSim2/src/spinSystem.cpp:483-745, restated by the oracle and pinned to the
    reference's own grid by the golden fixture): the cell counts and every
    list in the reference's order, for fibers along all three axes with radii
    that reach the halo lines on both sides; a grid whose fullest cell exceeds
    the reference's list capacity is refused as its build() refuses it."""
    from dsim_gb300.engine import Cylinders
    rng = np.random.default_rng(seed)
    fp = np.zeros((nfib, 4), np.float32)
    fp[:, :3] = rng.uniform(-1.0 + rmax, 1.0 - rmax, (nfib, 3)).astype(np.float32)
    axis = rng.integers(0, 3, nfib)
    fp[np.arange(nfib), axis] = 2.0
    r = (rng.uniform(0.3, 1.0, nfib) * rmax).astype(np.float32)
    fp[:, 3] = r * r
    maxR = float(r.max())
    fp = fp.reshape(-1)
    L = O.lib()
    geom = np.zeros(2, np.uint32)
    cl = C.c_float(0)
    L.or2_build_grid(nfib, fp, maxR, geom, C.byref(cl), None, None)
    n, maxfpc = int(geom[0]), int(geom[1])
    cc = np.zeros(n ** 3, np.uint32)
    cubes = np.zeros(max(1, n ** 3 * maxfpc), np.uint32)
    rc = L.or2_build_grid(nfib, fp, maxR, geom, C.byref(cl), cc, cubes)
    if rc != 0:
        with pytest.raises(Exception):
            Cylinders.from_arrays(fp, maxR)
        return
    c = Cylinders.from_arrays(fp, maxR)
    assert (c.numCubes, c.maxFPC, np.float32(c.cubeLength)) == (n, maxfpc, np.float32(cl.value))
    gcc, gcubes, gfp = c.grid()
    assert cc.sum() > nfib                          # halo lines were added
    assert np.array_equal(gcc, cc)
    assert np.array_equal(gcubes, cubes)
    assert np.array_equal(gfp.view(np.uint32), fp.view(np.uint32))
