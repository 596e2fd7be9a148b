"""Sharding a job's spins (the multi-GPU form) reproduces the unsharded run:
each shard sets its first spin's global index as its Philox spin base, so two
shards run one after another on one GPU give bit-identical per-spin states,
and their combined FP64 sums give the same signal."""
import numpy as np
import pytest

from scenarios import CylCase, MeshCase

pytestmark = pytest.mark.gpu


def test_mesh_shards_equal_one_run(engine, tmp_path):
    from dsim_gb300.engine import Mesh, Spins, mesh_params, mesh_run
    from dsim_gb300.replicas import shard, signal
    case = MeshCase(tmp_path, membranes="AM", permeability=0.05, N=1500)
    m = Mesh.load(case.path, case.spaceScale)
    p = mesh_params(case.stdDevs, case.T2, case.permeability, case.dt, case.pc)

    def run(lo, hi):
        s = Spins(hi - lo)
        s.set_spin_base(lo)
        s.set(case.pos.reshape(-1, 3)[lo:hi], case.mag[lo:hi], case.phase[lo:hi], case.comp[lo:hi],
              case.fiber[lo:hi])
        mesh_run(m, s, p, g=case.g, iterations=40, seed=5, count=True)
        return s.get(), s.signal(), s.counts()

    full, fsum, fcnt = run(0, case.N)
    parts = [run(*shard(case.N, r, 2)) for r in range(2)]
    for k in range(5):
        joined = np.concatenate([pt[0][k] for pt in parts])
        assert np.array_equal(joined.view(np.uint8), full[k].view(np.uint8))
    assert np.array_equal(np.concatenate([pt[2] for pt in parts]), fcnt)
    combined = sum(pt[1] for pt in parts)
    assert np.allclose(signal(combined), signal(fsum), rtol=1e-12)


def test_cylinder_shards_equal_one_run(engine, tmp_path):
    from dsim_gb300.engine import Cylinders, Spins, cyl_params, cyl_run
    from dsim_gb300.replicas import shard
    case = CylCase(tmp_path, permeability=0.02, inner=0.7, N=1200)
    c = Cylinders.load(case.path, case.spaceScale)
    p = cyl_params(case.D, case.D, 0.1 * case.D, case.spaceScale, 70.0, 8.0, 80.0, case.permeability,
                   case.inner, case.dt, case.pc)
    imo = np.full(case.N, 2, np.uint32)

    def run(lo, hi):
        s = Spins(hi - lo)
        s.set_spin_base(lo)
        s.set_cyl(case.pos.reshape(-1, 3)[lo:hi], None, None, imo[lo:hi], None)
        cyl_run(c, s, p, g=case.g, iterations=60, seed=8)
        return s.get_cyl()

    full = run(0, case.N)
    parts = [run(*shard(case.N, r, 3)) for r in range(3)]
    for k in range(4):
        joined = np.concatenate([pt[k] for pt in parts])
        assert np.array_equal(joined.view(np.uint8), full[k].view(np.uint8))
