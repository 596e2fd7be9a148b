"""GPU parity of the triangle-mesh hot path against the CPU oracle.

Replay mode feeds the same step stream to the GPU kernel and to the oracle
(the C restatement of dSim3's cpuIntegrate, pinned to the reference by the
golden fixtures): per-spin collision counts, positions, magnitude and phase
must agree bit for bit, compartments and fibers exactly.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from scenarios import MeshCase, draws

pytestmark = pytest.mark.gpu


def _oracle_run(case, mesh_o, cc, tic, maxtpc, iters, d, perm=None):
    p = O.params3(case.stdDevs, case.T2, case.permeability if perm is None else perm, case.dt, 50,
                  maxtpc)
    pos = case.pos.copy(); seed = np.zeros(2 * case.N, np.uint32)
    mag = case.mag.copy(); ph = case.phase.copy(); comp = case.comp.copy(); fib = case.fiber.copy()
    cnt = np.zeros(2 * case.N, np.uint32)
    capped, _ = O.integrate3(p, pos, seed, mag, ph, comp, fib, mesh_o.vertices, mesh_o.helpers,
                             mesh_o.triInfo, cc, tic, case.g, case.pc, iters, draws=d, counts=cnt)
    assert capped == 0
    return pos, mag, ph, comp, fib, cnt.reshape(-1, 2)


@pytest.mark.parametrize("membranes", ["AM", "G"])
def test_grid_build_matches_reference_membership(engine, tmp_path, membranes):
    from dsim_gb300.engine import Mesh
    case = MeshCase(tmp_path, membranes=membranes)
    m = Mesh.load(case.path, case.spaceScale)
    mo = O.Mesh(case.path, case.spaceScale)
    v, ti = m.arrays()
    assert np.array_equal(v.view(np.uint32), mo.vertices.view(np.uint32))
    assert np.array_equal(ti, mo.triInfo)
    cc, tic, maxtpc = O.populate_cubes(mo.vertices, mo.trgls, 50)
    start, tri = m.grid()
    counts = np.diff(start.astype(np.int64))
    assert np.array_equal(counts, cc.astype(np.int64))
    assert m.max_per_cell == maxtpc
    dense = tic.reshape(-1, maxtpc)
    for c in np.nonzero(cc)[0]:
        assert np.array_equal(tri[start[c]:start[c + 1]], dense[c, :cc[c]])


@pytest.mark.parametrize("membranes,perm,accel,sort,kernel,records", [
    ("AM", 0.05, None, 20, None, None), ("G", 0.0, None, 20, None, None),
    ("G", 0.3, None, 7, None, None), ("AM", 0.05, 13, 0, None, None),
    ("AM", 0.05, 37, 7, None, 16), ("AM", 0.05, 300, 0, None, None), ("G", 0.3, 13, 1, None, 16),
    ("AM", 0.05, None, 20, 7, None), ("AM", 0.05, None, 20, 6, 16), ("AM", 0.05, 75, 20, 7, None),
    ("AM", 0.05, None, 20, 5, None), ("G", 0.3, 37, 7, 6, 16), ("AM", 0.05, 300, 0, 5, None),
    ("G", 0.0, 75, 20, 5, 16), ("G", 0.3, None, 7, 7, None), ("AM", 0.05, 100, 20, 7, None),
    ("AM", 0.05, None, 20, None, 64), ("G", 0.3, 37, 7, 5, 64), ("AM", 0.05, 300, 0, 7, 64),
    ("G", 0.3, 13, 1, 6, 64), ("AM", 0.05, None, 20, 8, None), ("G", 0.3, 37, 7, 8, None),
    ("G", 0.0, 300, 0, 8, None), ("AM", 0.05, None, 20, 9, None), ("G", 0.3, 37, 7, 9, None),
    ("AM", 0.05, 300, 0, 9, None), ("G", 0.3, 1, 0, 9, None)])
def test_mesh_replay_bit_parity_native(engine, tmp_path, membranes, perm, accel, sort, kernel, records):
    """accel None: default fine grid; other: fine cells per axis (coarser and
    finer than the reference grid; 1: one cell, every triangle in one list).
    sort: steps between spin reorderings (0 = never).  kernel: step kernel
    variant (5, 6, 7: 8, 6, 4 blocks per SM; 8: records past the plane test
    queued and finished 32 at a time; 9: each cell's records staged in shared
    memory by bulk copies; 8 and 9 on 32-byte records, kernel 6's path on the
    others); records: fine-grid record bytes."""
    from dsim_gb300.engine import Mesh, Spins, mesh_params, mesh_run
    case = MeshCase(tmp_path, membranes=membranes, permeability=perm, N=1500)
    iters = 60
    d = draws(iters, case.N, seed=11)
    mo = O.Mesh(case.path, case.spaceScale)
    cc, tic, maxtpc = O.populate_cubes(mo.vertices, mo.trgls, 50)
    ref = _oracle_run(case, mo, cc, tic, maxtpc, iters, d)

    m = Mesh.load(case.path, case.spaceScale)
    if accel is not None:
        m.set_accel(accel)
    if records is not None:
        m.set_records(records)
    if kernel is not None:
        m.set_kernel(kernel)
    s = Spins(case.N)
    s.set_sort_interval(sort)
    s.set(case.pos, case.mag, case.phase, case.comp, case.fiber)
    p = mesh_params(case.stdDevs, case.T2, case.permeability, case.dt, case.pc)
    # two launches of 30 steps: state round-trips through HBM between calls
    mesh_run(m, s, p, g=case.g, iterations=30, draws=d[:30], count=True)
    mesh_run(m, s, p, g=case.g, iterations=30, draws=d[30:], count=True)
    pos, mag, ph, comp, fib = s.get()
    cnt = s.counts()
    assert s.status() == 0
    assert cnt.sum() > 0, "scenario produced no collisions"
    assert np.array_equal(cnt, ref[5]), "collision counts differ"
    assert np.array_equal(pos.view(np.uint32), ref[0].view(np.uint32))
    assert np.array_equal(mag.view(np.uint32), ref[1].view(np.uint32))
    assert np.array_equal(ph.view(np.uint32), ref[2].view(np.uint32))
    assert np.array_equal(comp, ref[3])
    assert np.array_equal(fib, ref[4])
    if perm > 0:
        assert cnt[:, 1].sum() > 0, "no permeation exercised"


def test_mesh_replay_bit_parity_dsim3_abi(engine, tmp_path):
    """Same replay through the reference-facing C-ABI (libdsim3.so), driven
    the way SpinSystem drives spinSystem.cuh: allocateArray / copy / bind /
    copyConstantToDevice by symbol name / integrateSystem."""
    from dsim_gb300 import _lib
    L = _lib.abi3()
    case = MeshCase(tmp_path, membranes="AM", permeability=0.05, N=1200)
    iters = 40
    d = draws(iters, case.N, seed=3)
    mo = O.Mesh(case.path, case.spaceScale)
    cc, tic, maxtpc = O.populate_cubes(mo.vertices, mo.trgls, 50)
    ref = _oracle_run(case, mo, cc, tic, maxtpc, iters, d)

    def dev(arr):
        p = C.c_void_p()
        L.allocateArray(C.byref(p), arr.nbytes)
        L.copyArrayToDevice(p, arr.ctypes.data, 0, arr.nbytes)
        return p

    dV, dH, dTI = dev(mo.vertices), dev(mo.helpers), dev(mo.triInfo)
    L.bindVertices(dV, len(mo.vertices))
    L.bindTriangleHelpers(dH, len(mo.helpers))
    L.bindTriInfo(dTI, len(mo.triInfo))
    dTic, dCc = dev(np.ascontiguousarray(tic)), dev(cc)
    for name, val, ty in (("k_numCubes", 50, np.uint32), ("k_totalNumCubes", 50 ** 3, np.uint32),
                          ("k_maxTrianglesPerCube", maxtpc, np.uint32),
                          ("k_cubeLength", np.float32(2.0) / np.float32(50), np.float32),
                          ("k_reflectionType", 1, np.uint32), ("k_permeability", case.permeability, np.float32),
                          ("k_deltaTime", case.dt, np.float32)):
        a = np.array([val], ty)
        L.copyConstantToDevice(name.encode(), a.ctypes.data, 0, 4)
    # T2 and sigma tables: the reference passes the address of a device pointer
    for name, tab in (("k_T2Values", case.T2), ("k_stdDevs", case.stdDevs)):
        dp = dev(np.ascontiguousarray(tab, np.float32))
        holder = C.c_void_p(dp.value)
        L.copyConstantToDevice(name.encode(), C.addressof(holder), 0, 4)
    spins = np.zeros(case.N, np.dtype([("mag", "<f4"), ("phase", "<f4"), ("comp", "u1"),
                                        ("pad", "u1"), ("fiber", "<u2")]))
    spins["mag"], spins["phase"], spins["comp"], spins["fiber"] = case.mag, case.phase, case.comp, case.fiber
    dPos, dSeed, dSpins = dev(case.pos.copy()), dev(np.zeros(2 * case.N, np.uint32)), dev(spins)
    dDraws = dev(d.reshape(-1))
    dCnt = dev(np.zeros(2 * case.N, np.uint32))
    L.dsim3_set_replay(dDraws, dCnt)
    g = _lib.Float3(*[float(x) for x in case.g])
    L.integrateSystem(dPos, dSeed, dSpins, float(case.dt), float(case.permeability), case.N, g,
                      float(case.pc), iters, dTic, dCc)
    L.dsim3_set_replay(None, None)
    assert L.dsim3_last_status() == 0, L.dsim3_last_error()
    pos = np.zeros_like(case.pos)
    out = np.zeros_like(spins)
    cnt = np.zeros(2 * case.N, np.uint32)
    L.copyArrayFromDevice(pos.ctypes.data, dPos, 0, pos.nbytes)
    L.copyArrayFromDevice(out.ctypes.data, dSpins, 0, out.nbytes)
    L.copyArrayFromDevice(cnt.ctypes.data, dCnt, 0, cnt.nbytes)
    assert L.dsim3_status() == 0
    assert np.array_equal(cnt.reshape(-1, 2), ref[5])
    assert np.array_equal(pos.view(np.uint32), ref[0].view(np.uint32))
    assert np.array_equal(out["mag"].view(np.uint32), ref[1].view(np.uint32))
    assert np.array_equal(out["phase"].view(np.uint32), ref[2].view(np.uint32))
    assert np.array_equal(out["comp"], ref[3])
    assert np.array_equal(out["fiber"], ref[4])
    for p in (dV, dH, dTI, dTic, dCc, dPos, dSeed, dSpins, dDraws, dCnt):
        L.freeArray(p)


def test_mesh_philox_run_is_deterministic_and_in_box(engine, tmp_path):
    from dsim_gb300.engine import Mesh, Spins, mesh_params, mesh_run
    case = MeshCase(tmp_path, membranes="AM", permeability=0.01, N=4096)
    m = Mesh.load(case.path, case.spaceScale)
    p = mesh_params(case.stdDevs, case.T2, case.permeability, case.dt, case.pc)
    outs = []
    for _ in range(2):
        s = Spins(case.N)
        s.set(case.pos, case.mag, case.phase, case.comp, case.fiber)
        mesh_run(m, s, p, g=case.g, iterations=200, seed=1234, step0=0, count=True)
        outs.append(s.get())
        assert s.status() == 0
        assert s.counts().sum() > 0
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)
    pos = outs[0][0]
    assert np.all(np.abs(pos) <= np.float32(0.995))


@pytest.mark.parametrize("cap,refl", [(1, 1), (2, 1), (2, 0)])
def test_mesh_replay_parity_at_the_subsegment_cap(engine, tmp_path, cap, refl):
    """The reference's sub-segment loop has no bound (a spin caught between
    two intersecting membranes would loop forever); the engine stops a step
    after `maxSubsegments` hits, leaves the spin at the start of its current
    sub-segment (the last hit point) and raises status bit 1.  With a cap of
    1 or 2 most colliding steps end there: the oracle, given the same cap,
    agrees bit for bit.  refl 0: the reference's return-to-start reflection."""
    from dsim_gb300.engine import Mesh, Spins, mesh_params, mesh_run
    case = MeshCase(tmp_path, membranes="AM", permeability=0.05, N=1500)
    iters = 40
    d = draws(iters, case.N, seed=17)
    mo = O.Mesh(case.path, case.spaceScale)
    cc, tic, maxtpc = O.populate_cubes(mo.vertices, mo.trgls, 50)
    p = O.params3(case.stdDevs, case.T2, case.permeability, case.dt, 50, maxtpc, reflectionType=refl,
                  maxSubsegments=cap)
    pos = case.pos.copy(); seed = np.zeros(2 * case.N, np.uint32)
    mag = case.mag.copy(); ph = case.phase.copy(); comp = case.comp.copy(); fib = case.fiber.copy()
    cnt = np.zeros(2 * case.N, np.uint32)
    capped, _ = O.integrate3(p, pos, seed, mag, ph, comp, fib, mo.vertices, mo.helpers, mo.triInfo, cc, tic,
                             case.g, case.pc, iters, draws=d, counts=cnt)
    assert capped > 0
    m = Mesh.load(case.path, case.spaceScale)
    s = Spins(case.N)
    s.set(case.pos, case.mag, case.phase, case.comp, case.fiber)
    gp = mesh_params(case.stdDevs, case.T2, case.permeability, case.dt, case.pc, reflectionType=refl,
                     maxSubsegments=cap)
    mesh_run(m, s, gp, g=case.g, iterations=iters, draws=d, count=True)
    gpos, gmag, gph, gcomp, gfib = s.get()
    assert s.status() & 1
    assert np.array_equal(s.counts(), cnt.reshape(-1, 2))
    assert np.array_equal(gpos.view(np.uint32), pos.view(np.uint32))
    assert np.array_equal(gph.view(np.uint32), ph.view(np.uint32))
    assert np.array_equal(gcomp, comp) and np.array_equal(gfib, fib)


def test_mesh_dsim3_abi_arrays_rewritten_in_place(engine, tmp_path):
    """Between two integrateSystem calls the caller overwrites vertices,
    helpers, triInfo and the grid in the same device arrays (the same sizes
    and constants): the second call must walk the new mesh, bit for bit with
    the oracle run on the two meshes in turn.  The drop-in notices the change
    from the arrays' contents, not their addresses."""
    from dsim_gb300 import _lib
    from dsim_gb300 import substrates as S
    L = _lib.abi3()
    case = MeshCase(tmp_path, membranes="AM", permeability=0.05, N=1500)
    tube2 = dict(case.tube)
    tube2["vertices"] = (case.tube["vertices"] + np.array([0.6, -0.35, 0.2], np.float32)).astype(np.float32)
    path2 = str(tmp_path / "mesh_shifted.txt")
    S.write_mesh_file(path2, tube2)
    meshes = []
    for pth in (case.path, path2):
        mo = O.Mesh(pth, case.spaceScale)
        cc, tic, maxtpc = O.populate_cubes(mo.vertices, mo.trgls, 50)
        meshes.append((mo, cc, tic.reshape(-1, maxtpc), maxtpc))
    W = max(m[3] for m in meshes)
    dense = []
    for mo, cc, tic, maxtpc in meshes:
        t = np.zeros((50 ** 3, W), np.uint32)
        t[:, :maxtpc] = tic
        dense.append(np.ascontiguousarray(t.reshape(-1)))
    assert not np.array_equal(meshes[0][0].vertices, meshes[1][0].vertices)
    it1, it2 = 30, 30
    d = draws(it1 + it2, case.N, seed=23)
    p = O.params3(case.stdDevs, case.T2, case.permeability, case.dt, 50, W)
    pos = case.pos.copy(); seed = np.zeros(2 * case.N, np.uint32)
    mag = case.mag.copy(); ph = case.phase.copy(); comp = case.comp.copy(); fib = case.fiber.copy()
    cnt = np.zeros(2 * case.N, np.uint32)
    for (mo, cc, _, _), t, dd in ((meshes[0], dense[0], d[:it1]), (meshes[1], dense[1], d[it1:])):
        capped, _ = O.integrate3(p, pos, seed, mag, ph, comp, fib, mo.vertices, mo.helpers, mo.triInfo, cc, t,
                                 case.g, case.pc, len(dd), draws=dd, counts=cnt)
        assert capped == 0
    bufs = []

    def dev(arr):
        q = C.c_void_p()
        L.allocateArray(C.byref(q), arr.nbytes)
        L.copyArrayToDevice(q, arr.ctypes.data, 0, arr.nbytes)
        bufs.append(q)
        return q

    try:
        mo0, cc0 = meshes[0][0], meshes[0][1]
        dV, dH, dTI = dev(mo0.vertices), dev(mo0.helpers), dev(mo0.triInfo)
        dTic, dCc = dev(dense[0]), dev(cc0)
        L.bindVertices(dV, len(mo0.vertices))
        L.bindTriangleHelpers(dH, len(mo0.helpers))
        L.bindTriInfo(dTI, len(mo0.triInfo))
        for name, val, ty in (("k_numCubes", 50, np.uint32), ("k_totalNumCubes", 50 ** 3, np.uint32),
                              ("k_maxTrianglesPerCube", W, np.uint32),
                              ("k_cubeLength", np.float32(2.0) / np.float32(50), np.float32),
                              ("k_reflectionType", 1, np.uint32), ("k_permeability", case.permeability, np.float32),
                              ("k_deltaTime", case.dt, np.float32)):
            a = np.array([val], ty)
            L.copyConstantToDevice(name.encode(), a.ctypes.data, 0, 4)
        for name, tab in (("k_T2Values", case.T2), ("k_stdDevs", case.stdDevs)):
            a = np.ascontiguousarray(tab, np.float32)
            L.copyConstantToDevice(name.encode(), a.ctypes.data, 0, 16)
        spins = np.zeros(case.N, np.dtype([("mag", "<f4"), ("phase", "<f4"), ("comp", "u1"), ("pad", "u1"),
                                            ("fiber", "<u2")]))
        spins["mag"], spins["phase"], spins["comp"], spins["fiber"] = case.mag, case.phase, case.comp, case.fiber
        dPos, dSeed, dSpins = dev(case.pos.copy()), dev(np.zeros(2 * case.N, np.uint32)), dev(spins)
        dD1, dD2 = dev(np.ascontiguousarray(d[:it1]).reshape(-1)), dev(np.ascontiguousarray(d[it1:]).reshape(-1))
        dCnt = dev(np.zeros(2 * case.N, np.uint32))
        g = _lib.Float3(*[float(x) for x in case.g])
        for seg, (dd, its) in enumerate(((dD1, it1), (dD2, it2))):
            if seg:
                mo1, cc1 = meshes[1][0], meshes[1][1]
                for dst, src in ((dV, mo1.vertices), (dH, mo1.helpers), (dTI, mo1.triInfo), (dTic, dense[1]),
                                 (dCc, cc1)):
                    L.copyArrayToDevice(dst, src.ctypes.data, 0, src.nbytes)
            L.dsim3_set_replay(dd, dCnt)
            L.integrateSystem(dPos, dSeed, dSpins, float(case.dt), float(case.permeability), case.N, g,
                              float(case.pc), its, dTic, dCc)
            L.dsim3_set_replay(None, None)
            assert L.dsim3_last_status() == 0, L.dsim3_last_error()
        gpos = np.zeros_like(case.pos)
        out = np.zeros_like(spins)
        gcnt = np.zeros(2 * case.N, np.uint32)
        L.copyArrayFromDevice(gpos.ctypes.data, dPos, 0, gpos.nbytes)
        L.copyArrayFromDevice(out.ctypes.data, dSpins, 0, out.nbytes)
        L.copyArrayFromDevice(gcnt.ctypes.data, dCnt, 0, gcnt.nbytes)
        assert L.dsim3_status() == 0
        assert np.array_equal(gcnt, cnt)
        assert np.array_equal(gpos.view(np.uint32), pos.view(np.uint32))
        assert np.array_equal(out["phase"].view(np.uint32), ph.view(np.uint32))
        assert np.array_equal(out["mag"].view(np.uint32), mag.view(np.uint32))
        assert np.array_equal(out["comp"], comp) and np.array_equal(out["fiber"], fib)
    finally:
        for q in bufs:
            L.freeArray(q)
