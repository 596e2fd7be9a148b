"""Edge cases of the mesh step against the oracle, and a size-independent
property at the full mesh size.

* A single spin and a ragged count (33) in replay mode, bit for bit.
* Spins placed exactly on reference-cell boundaries (x = -1 + k L) and on
  fine-cell boundaries, where the cell of a point and the first cell of the
  reference's walk are decided by floor of an exact multiple.
* Spins at the clamp (+-0.995) with steps pushing them out of the box.
* Cylinders: spins on grid-cell boundaries, on cylinder surfaces and at the
  clamp, bit for bit against the dSim2 oracle.
* At the full C2 size (2.56M triangles, 1M spins), every step kernel variant
  gives the same positions, phases and collision counts bit for bit, every
  position stays within the clamp, and the counts are nonzero.
"""
import numpy as np
import pytest

import oracle as O
from scenarios import MeshCase, draws

pytestmark = pytest.mark.gpu
F = np.float32


def _replay(case, pos, iters, seed):
    """GPU replay through dsim_mesh_run and the oracle on the same draws."""
    from dsim_gb300.engine import Mesh, Spins, mesh_params, mesh_run
    pos = np.ascontiguousarray(pos, F).reshape(-1, 3)
    N = len(pos)
    comp, fib = case._compartments(pos, "AM")
    d = draws(iters, N, seed=seed)
    mo = O.Mesh(case.path, case.spaceScale)
    cc, tic, maxtpc = O.populate_cubes(mo.vertices, mo.trgls, 50)
    p = O.params3(case.stdDevs, case.T2, case.permeability, case.dt, 50, maxtpc)
    rp = pos.reshape(-1).copy(); seed0 = np.zeros(2 * N, np.uint32)
    rmag = np.ones(N, F); rph = np.zeros(N, F); rcomp = comp.copy(); rfib = fib.copy()
    cnt = np.zeros(2 * N, np.uint32)
    capped, _ = O.integrate3(p, rp, seed0, rmag, rph, rcomp, rfib, mo.vertices, mo.helpers, mo.triInfo, cc, tic,
                             case.g, case.pc, iters, draws=d, counts=cnt)
    assert capped == 0
    m = Mesh.load(case.path, case.spaceScale)
    s = Spins(N)
    s.set(pos.reshape(-1), np.ones(N, F), np.zeros(N, F), comp, fib)
    gp = mesh_params(case.stdDevs, case.T2, case.permeability, case.dt, case.pc)
    mesh_run(m, s, gp, g=case.g, iterations=iters, draws=d, count=True)
    assert s.status() == 0
    gpos, gmag, gph, gcomp, gfib = s.get()
    assert np.array_equal(s.counts(), cnt.reshape(-1, 2))
    assert np.array_equal(gpos.view(np.uint32), rp.view(np.uint32))
    assert np.array_equal(gmag.view(np.uint32), rmag.view(np.uint32))
    assert np.array_equal(gph.view(np.uint32), rph.view(np.uint32))
    assert np.array_equal(gcomp, rcomp) and np.array_equal(gfib, rfib)
    return cnt.reshape(-1, 2)


@pytest.mark.parametrize("N", [1, 33])
def test_tiny_and_ragged_spin_counts(engine, tmp_path, N):
    case = MeshCase(tmp_path, membranes="AM", permeability=0.05, N=1500)
    pos = case.pos.reshape(-1, 3)[:N]
    _replay(case, pos, 80, seed=21 + N)


def test_spins_on_cell_boundaries(engine, tmp_path):
    """x, y, z exactly on reference-cell boundaries -1 + k (2/50) and on
    fine-cell boundaries -1 + k (2/112), in float."""
    case = MeshCase(tmp_path, membranes="AM", permeability=0.05, N=1500)
    rng = np.random.default_rng(3)
    k = rng.integers(3, 47, (600, 3))
    ref = (F(-1.0) + k.astype(F) * (F(2.0) / F(50))).astype(F)
    kf = rng.integers(8, 105, (600, 3))
    fine = (F(-1.0) + kf.astype(F) * (F(2.0) / F(112))).astype(F)
    mixed = ref.copy()
    mixed[:, 1] = rng.uniform(-0.9, 0.9, 600).astype(F)   # one coordinate free
    pos = np.concatenate([ref, fine, mixed]).astype(F)
    cnt = _replay(case, pos, 60, seed=5)
    assert cnt.sum() > 0


def test_spins_at_the_clamp(engine, tmp_path):
    """Spins at +-0.995 on each face, edge and corner of the box, stepping
    outward and back: the clamp of cpuIntegrate (x > 1 - r -> 1 - r)."""
    case = MeshCase(tmp_path, membranes="AM", permeability=0.05, N=1500)
    rng = np.random.default_rng(4)
    pos = rng.uniform(-0.9, 0.9, (900, 3)).astype(F)
    c = F(0.995)
    for i in range(900):
        face = rng.integers(0, 3, rng.integers(1, 4))
        for a in face:
            pos[i, a] = c if rng.random() < 0.5 else -c
    _replay(case, pos, 60, seed=6)


def test_full_size_variants_agree(engine):
    """Bench-size mesh: all step kernel variants, one 20-step call on 1M spins."""
    import bench
    from dsim_gb300.engine import Spins, mesh_run
    W = bench.Workload(axons=400, spins=1 << 20, seed=1)
    m = bench.make_mesh(W)
    p = bench.mesh_params_of(W)
    outs = {}
    for k in (6, 5, 7, 8, 9):
        m.set_kernel(k)
        s = Spins(W.N)
        s.set(W.pos, np.ones(W.N, F), np.zeros(W.N, F), W.comp, W.fiber)
        mesh_run(m, s, p, grad_per_step=W.grad[:20], iterations=20, seed=9, step0=0, count=True)
        assert s.status() == 0
        pos, mag, ph, comp, fib = s.get()
        outs[k] = (pos, ph, comp, s.counts())
        del s
    pos6, ph6, comp6, cnt6 = outs[6]
    assert cnt6[:, 0].sum() > 0
    assert np.all(np.abs(pos6) <= F(0.995))
    for k, (pos, ph, comp, cnt) in outs.items():
        assert np.array_equal(pos.view(np.uint32), pos6.view(np.uint32)), k
        assert np.array_equal(ph.view(np.uint32), ph6.view(np.uint32)), k
        assert np.array_equal(comp, comp6) and np.array_equal(cnt, cnt6), k
    m.set_kernel(6)


def test_cylinder_edges(engine, tmp_path):
    """Cylinders: spins on the grid's cell boundaries, on cylinder surfaces
    (centre + r (cos, sin), in float) and at the clamp, with permeable
    myelin; replay parity with the dSim2 oracle."""
    from dsim_gb300.engine import Cylinders, Spins, cyl_params, cyl_run
    from scenarios import CylCase
    from test_gpu_cyl import _oracle, _setup
    case = CylCase(tmp_path, permeability=0.05, inner=0.7, N=3000)
    fp, maxR = O.load_fibers2(case.path, case.spaceScale)
    _, _, n, _, L = O.build_grid2(fp, maxR)
    rng = np.random.default_rng(8)
    k = rng.integers(0, n + 1, (1000, 3))
    on_cells = (F(-1.0) + k.astype(F) * F(L)).astype(F)
    on_cells = np.clip(on_cells, F(-0.995), F(0.995))
    f4 = fp.reshape(-1, 4)
    sel = rng.integers(0, len(f4), 1000)
    ang = rng.uniform(0, 2 * np.pi, 1000)
    r = np.sqrt(f4[sel, 3]).astype(F)
    surf = np.zeros((1000, 3), F)
    surf[:, 0] = f4[sel, 0] + r * np.cos(ang).astype(F)
    surf[:, 1] = f4[sel, 1] + r * np.sin(ang).astype(F)
    surf[:, 2] = rng.uniform(-0.9, 0.9, 1000).astype(F)
    surf = np.clip(surf, F(-0.995), F(0.995))
    clamp = rng.uniform(-0.9, 0.9, (1000, 3)).astype(F)
    for i in range(1000):
        for a in rng.integers(0, 3, rng.integers(1, 4)):
            clamp[i, a] = F(0.995) if rng.random() < 0.5 else F(-0.995)
    case.pos = np.concatenate([on_cells, surf, clamp]).astype(F).reshape(-1)
    case.N = 3000
    fp, maxR, cc, cubes, n, maxfpc, L, near, imo = _setup(case)
    iters = 60
    d = draws(iters, case.N, seed=23)
    rpos, rpar, rcnt = _oracle(case, fp, cc, cubes, n, maxfpc, L, iters, d, near, imo)
    c = Cylinders.load(case.path, case.spaceScale)
    s = Spins(case.N)
    s.set_cyl(case.pos, None, None, imo, near)
    p = cyl_params(case.D, case.D, 0.1 * case.D, case.spaceScale, 70.0, 8.0, 80.0, case.permeability,
                   case.inner, case.dt, case.pc)
    cyl_run(c, s, p, g=case.g, iterations=iters, draws=d, count=True)
    pos, mag, ph, gimo, gnear = s.get_cyl()
    assert s.status() == 0
    assert s.counts().sum() > 0
    assert np.array_equal(s.counts(), rcnt)
    assert np.array_equal(pos.reshape(-1, 3).view(np.uint32), rpos[:, :3].view(np.uint32))
    assert np.array_equal(ph.view(np.uint32), rpar[:, 1].view(np.uint32))
    assert np.array_equal(gimo, rpar[:, 3].astype(np.uint32))
