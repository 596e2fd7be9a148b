"""Bit parity with the oracle at the size of the headline mesh workload.

The workload of bench.py: 400 beaded tubes, 2,560,000 triangles in a 50 um
cube (spaceScale 25, the reference's 50^3 grid of 1 um cells, up to 256
triangles per cell, overlapping tubes).  Its first 4,096 spins (the spins of
the 1,048,576-spin workload are drawn in order from one seeded stream, so
these are exactly its first 4,096) walk 300 replayed steps:

* through dsim_mesh_run with the default step kernel and fine grid, on the
  mesh the bench builds from arrays;
* through libdsim3.so integrateSystem with dsim3_set_replay, on the arrays
  the reference's host code would bind (initFibers and populateCubes as the
  oracle restates them), with and without permeation.

Every per-spin collision count, position, magnitude, phase, compartment and
fiber must equal the oracle's (or3_integrate on its own populateCubes grid,
dSim3/src/spinKernelCpu.cpp:198-301, 430-499) bit for bit.
"""
import ctypes as C
import os
import sys

import numpy as np
import pytest

import oracle as O
from scenarios import draws

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ITERS = 300


@pytest.fixture(scope="module")
def full(tmp_path_factory):
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench
    from dsim_gb300 import substrates as S
    W = bench.Workload(axons=400, spins=4096, seed=1)
    assert len(W.tube["trgls"]) == 2_560_000
    path = str(tmp_path_factory.mktemp("full") / "workload.mesh")
    S.write_mesh_file(path, W.tube)
    mo = O.Mesh(path, W.spaceScale)
    cc, tic, maxtpc = O.populate_cubes(mo.vertices, mo.trgls, W.numCubes)
    return W, mo, cc, tic, maxtpc


def _oracle(W, mo, cc, tic, maxtpc, perm, d):
    p = O.params3(W.stdDevs, W.T2, perm, W.dt, W.numCubes, maxtpc)
    N = W.N
    pos = W.pos.copy(); seed = np.zeros(2 * N, np.uint32)
    mag = np.ones(N, np.float32); ph = np.zeros(N, np.float32)
    comp = W.comp.copy(); fib = W.fiber.copy()
    cnt = np.zeros(2 * N, np.uint32)
    capped, _ = O.integrate3(p, pos, seed, mag, ph, comp, fib, mo.vertices, mo.helpers, mo.triInfo, cc, tic,
                             W.g, W.pc, ITERS, draws=d, counts=cnt)
    assert capped == 0
    cnt = cnt.reshape(-1, 2)
    assert cnt[:, 0].sum() > 0
    return pos, mag, ph, comp, fib, cnt


def _same(got, ref):
    pos, mag, ph, comp, fib, cnt = got
    rpos, rmag, rph, rcomp, rfib, rcnt = ref
    assert np.array_equal(cnt, rcnt), np.nonzero((cnt != rcnt).any(1))[0][:10]
    assert np.array_equal(pos.view(np.uint32), rpos.view(np.uint32))
    assert np.array_equal(mag.view(np.uint32), rmag.view(np.uint32))
    assert np.array_equal(ph.view(np.uint32), rph.view(np.uint32))
    assert np.array_equal(comp, rcomp) and np.array_equal(fib, rfib)


def test_fullsize_native_run_bit_parity(engine, full):
    import bench
    from dsim_gb300.engine import Spins, mesh_run
    W, mo, cc, tic, maxtpc = full
    m = bench.make_mesh(W)                      # the bench's own mesh, default fine grid
    v, ti = m.arrays()
    assert np.array_equal(v.view(np.uint32), mo.vertices.view(np.uint32))
    assert np.array_equal(ti, mo.triInfo)
    assert m.max_per_cell == maxtpc
    d = draws(ITERS, W.N, seed=31)
    ref = _oracle(W, mo, cc, tic, maxtpc, 0.0, d)
    s = Spins(W.N)
    s.set(W.pos, np.ones(W.N, np.float32), np.zeros(W.N, np.float32), W.comp, W.fiber)
    mesh_run(m, s, bench.mesh_params_of(W), g=W.g, iterations=ITERS, draws=d, count=True)
    assert s.status() == 0
    _same(tuple(s.get()) + (s.counts(),), ref)


@pytest.mark.parametrize("perm", [0.0, 0.02])
def test_fullsize_dsim3_abi_bit_parity(engine, full, perm):
    from dsim_gb300 import _lib
    W, mo, cc, tic, maxtpc = full
    L = _lib.abi3()
    N = W.N
    d = draws(ITERS, N, seed=41)
    ref = _oracle(W, mo, cc, tic, maxtpc, perm, d)
    if perm > 0:
        assert ref[5][:, 1].sum() > 0
    bufs = []

    def dev(arr):
        p = C.c_void_p()
        L.allocateArray(C.byref(p), arr.nbytes)
        assert p.value
        L.copyArrayToDevice(p, arr.ctypes.data, 0, arr.nbytes)
        bufs.append(p)
        return p

    try:
        dV, dH, dTI = dev(mo.vertices), dev(mo.helpers), dev(mo.triInfo)
        L.bindVertices(dV, len(mo.vertices))
        L.bindTriangleHelpers(dH, len(mo.helpers))
        L.bindTriInfo(dTI, len(mo.triInfo))
        dTic, dCc = dev(np.ascontiguousarray(tic)), dev(cc)
        for name, val, ty in (("k_numCubes", W.numCubes, np.uint32), ("k_totalNumCubes", W.numCubes ** 3, np.uint32),
                              ("k_maxTrianglesPerCube", maxtpc, np.uint32),
                              ("k_cubeLength", np.float32(2.0) / np.float32(W.numCubes), np.float32),
                              ("k_reflectionType", 1, np.uint32), ("k_permeability", perm, np.float32),
                              ("k_deltaTime", W.dt, np.float32)):
            a = np.array([val], ty)
            L.copyConstantToDevice(name.encode(), a.ctypes.data, 0, 4)
        for name, tab in (("k_T2Values", W.T2), ("k_stdDevs", W.stdDevs)):
            a = np.ascontiguousarray(tab, np.float32)
            L.copyConstantToDevice(name.encode(), a.ctypes.data, 0, 16)
        spins = np.zeros(N, np.dtype([("mag", "<f4"), ("phase", "<f4"), ("comp", "u1"), ("pad", "u1"),
                                      ("fiber", "<u2")]))
        spins["mag"], spins["comp"], spins["fiber"] = 1.0, W.comp, W.fiber
        dPos, dSeed, dSpins = dev(W.pos.copy()), dev(np.zeros(2 * N, np.uint32)), dev(spins)
        dDraws, dCnt = dev(d.reshape(-1)), dev(np.zeros(2 * N, np.uint32))
        L.dsim3_set_replay(dDraws, dCnt)
        g = _lib.Float3(*[float(x) for x in W.g])
        L.integrateSystem(dPos, dSeed, dSpins, float(W.dt), float(perm), N, g, float(W.pc), ITERS, dTic, dCc)
        L.dsim3_set_replay(None, None)
        assert L.dsim3_last_status() == 0, L.dsim3_last_error()
        pos = np.zeros_like(W.pos)
        out = np.zeros_like(spins)
        cnt = np.zeros(2 * N, np.uint32)
        L.copyArrayFromDevice(pos.ctypes.data, dPos, 0, pos.nbytes)
        L.copyArrayFromDevice(out.ctypes.data, dSpins, 0, out.nbytes)
        L.copyArrayFromDevice(cnt.ctypes.data, dCnt, 0, cnt.nbytes)
        assert L.dsim3_status() == 0
        _same((pos, out["mag"].copy(), out["phase"].copy(), out["comp"].copy(), out["fiber"].copy(),
               cnt.reshape(-1, 2)), ref)
    finally:
        for p in bufs:
            L.freeArray(p)
