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


def test_cyl_replay_bit_parity_dsim2_abi(engine, tmp_path):
    """Replay through the reference-facing dSim2 C-ABI (libdsim2.so)."""
    from dsim_gb300 import _lib
    L2 = _lib.abi2()
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
