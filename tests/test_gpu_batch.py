"""The batching form (include/dsim_batch.h): many jobs in one step launch.

* A mesh job alone in a batch reproduces dsim_mesh_run with the same seed bit
  for bit (positions, magnitudes, compartments, collision totals), and its
  moment-based phase equals the plain run's float phase within 2e-5 relative
  to the largest phase.  The plain run is pinned to the oracle by
  test_gpu_mesh.py, so this chains the batch kernel to the reference.
* The same for a cylinder job against dsim_cyl_run.
* Every job's result is the same alone and in a mix of jobs (bit for bit per
  spin; FP64 signals within 1e-12), including jobs admitted while others run
  and after finished jobs are compacted away.
"""
import numpy as np
import pytest

import oracle as O
from scenarios import CylCase, MeshCase

pytestmark = pytest.mark.gpu
F = np.float32


def _mesh_job(case, steps, seed, delta=0.1, Delta=0.2):
    from dsim_gb300.engine import pgse_table
    w = pgse_table(steps, float(case.dt), delta, Delta)
    return dict(pos=case.pos, comp=case.comp, fiber=case.fiber.astype(np.uint32), steps=steps,
                dt=case.dt, step_sd=case.stdDevs, T2=case.T2, phase_constant=case.pc, seed=seed,
                permeability=case.permeability, waveform="table", table=w), w


def test_batch_mesh_job_matches_plain_run(engine, tmp_path):
    from dsim_gb300.engine import Batch, Mesh, Spins, mesh_params, mesh_run
    case = MeshCase(tmp_path, membranes="AM", permeability=0.05, N=1500)
    steps, seed = 60, 77
    job, w = _mesh_job(case, steps, seed)
    m = Mesh.load(case.path, case.spaceScale)
    s = Spins(case.N)
    s.set(case.pos, case.mag, np.zeros(case.N, F), case.comp, case.fiber)
    p = mesh_params(case.stdDevs, case.T2, case.permeability, case.dt, case.pc)
    gps = (w[:, None] * np.asarray(case.g, F)[None, :]).astype(F)
    mesh_run(m, s, p, grad_per_step=gps, iterations=steps, seed=seed, count=True)
    pos, mag, ph, comp, fib = s.get()
    cnt = s.counts()

    b = Batch(1 << 16, 16)
    b.configure(chunk=7, occupancy=4, graph_chunks=2)
    sid = b.add_mesh(m)
    jid = b.submit(sid, **job)
    b.run()
    assert b.status() == 0
    bpos, bmag, mom, bcomp, bfib = b.get(jid, case.N)
    assert np.array_equal(bpos.view(np.uint32), pos.view(np.uint32))
    assert np.array_equal(bmag.view(np.uint32), mag.view(np.uint32))
    assert np.array_equal(bcomp, comp)
    assert np.array_equal(bfib & 0xFFFF, fib.astype(np.uint32))
    assert np.array_equal(b.counts(jid), cnt.sum(axis=0).astype(np.uint64))
    M = mom[:, :3].astype(np.float64) - mom[:, 3:].astype(np.float64)
    phase = float(case.pc) * (M @ np.asarray(case.g, np.float64))
    assert np.abs(phase - ph).max() <= 2e-5 * max(1.0, np.abs(ph).max())
    # FP64 signal from the moments, against numpy on the same moments
    sig = b.signal(jid, np.asarray(case.g, F)[None, :])[0]
    want = np.array([np.sum(bmag * np.cos(phase)), np.sum(bmag * np.sin(phase)), case.N])
    assert np.allclose(sig[0], want, rtol=1e-9, atol=1e-9)


def test_batch_cyl_job_matches_plain_run(engine, tmp_path):
    from dsim_gb300.engine import Batch, Cylinders, Spins, cyl_params, cyl_run, pgse_table
    case = CylCase(tmp_path, permeability=0.05, inner=0.7, N=2000)
    fp, maxR = O.load_fibers2(case.path, case.spaceScale)
    cc, cubes, n, maxfpc, L = O.build_grid2(fp, maxR)
    near = np.zeros(case.N, np.uint32)
    imo = np.zeros(case.N, np.uint32)
    pos4 = np.zeros(4 * case.N, F)
    pos4.reshape(-1, 4)[:, :3] = case.pos.reshape(-1, 3)
    O.lib().or2_find_nearest(case.N, pos4, fp, n, L, maxfpc, cc, cubes, float(case.inner), near, imo)
    steps, seed = 70, 5
    c = Cylinders.load(case.path, case.spaceScale)
    s = Spins(case.N)
    s.set_cyl(case.pos, None, None, imo, near)
    p = cyl_params(case.D, case.D, 0.1 * case.D, case.spaceScale, 70.0, 8.0, 80.0, case.permeability,
                   case.inner, case.dt, case.pc)
    w = pgse_table(steps, float(case.dt), 0.2, 0.4)
    gps = (w[:, None] * np.asarray(case.g, F)[None, :]).astype(F)
    cyl_run(c, s, p, grad_per_step=gps, iterations=steps, seed=seed, count=True)
    pos, mag, ph, gimo, gnear = s.get_cyl()
    cnt = s.counts()

    ss = F(case.spaceScale)
    sd = [np.sqrt(F(2) * (F(adc) / (ss * ss)) * F(case.dt)) for adc in (case.D, 0.1 * case.D, case.D)]
    b = Batch(1 << 16, 16)
    b.configure(chunk=9, occupancy=4, graph_chunks=4)
    sid = b.add_cyl(c)
    jid = b.submit(sid, case.pos, imo.astype(np.uint8), near, steps, case.dt, sd + [0.0], [70.0, 8.0, 80.0, 0.0],
                   case.pc, seed, permeability=case.permeability, waveform="table", table=w,
                   inner_radius_proportion=case.inner)
    b.run()
    assert b.status() == 0
    bpos, bmag, mom, bimo, bnear = b.get(jid, case.N)
    assert np.array_equal(bpos.view(np.uint32), pos.view(np.uint32))
    assert np.array_equal(bmag.view(np.uint32), mag.view(np.uint32))
    assert np.array_equal(bimo.astype(np.uint32), gimo)
    inside = gimo < 2
    assert np.array_equal(bnear[inside], gnear[inside])
    assert np.array_equal(b.counts(jid), cnt.sum(axis=0).astype(np.uint64))
    M = mom[:, :3].astype(np.float64) - mom[:, 3:].astype(np.float64)
    phase = float(case.pc) * (M @ np.asarray(case.g, np.float64))
    assert np.abs(phase - ph).max() <= 2e-5 * max(1.0, np.abs(ph).max())


def _run_alone(m_by_name, c, jobs, names):
    from dsim_gb300.engine import Batch
    out = {}
    for name in names:
        kind, job, n = jobs[name]
        b = Batch(1 << 16, 4)
        b.configure(chunk=10, occupancy=4, graph_chunks=2)
        sid = b.add_mesh(m_by_name[kind]) if kind != "cyl" else b.add_cyl(c)
        jid = b.submit(sid, **job)
        b.run()
        out[name] = b.get(jid, n), b.signal(jid, np.array([[1e-3, 2e-3, 0.5e-3]], F)), b.counts(jid)
        b.close()
    return out


def test_batch_job_same_alone_and_in_mix(engine, tmp_path):
    from dsim_gb300.engine import Batch, Cylinders, Mesh
    am = MeshCase(tmp_path, membranes="AM", permeability=0.05, N=1000)
    gl = MeshCase(tmp_path, membranes="G", permeability=0.2, N=700, seed=4)
    cy = CylCase(tmp_path, permeability=0.02, inner=0.7, N=900)
    meshes = {"am": Mesh.load(am.path, am.spaceScale), "g": Mesh.load(gl.path, gl.spaceScale)}
    c = Cylinders.load(cy.path, cy.spaceScale)
    ja, _ = _mesh_job(am, 50, 11)
    jg, _ = _mesh_job(gl, 80, 12)
    jg["waveform"], jg["table"], jg["delta"], jg["Delta"] = "pgse", None, 0.15, 0.3
    ss = F(cy.spaceScale)
    sd = [float(np.sqrt(F(2) * (F(adc) / (ss * ss)) * F(cy.dt))) for adc in (2.0, 0.2, 2.0)] + [0.0]
    jc = dict(pos=cy.pos, comp=np.full(cy.N, 2, np.uint8), fiber=None, steps=40, dt=cy.dt, step_sd=sd,
              T2=[70.0, 8.0, 80.0, 0.0], phase_constant=cy.pc, seed=13, permeability=0.02,
              waveform="ogse", delta=0.2, Delta=0.25, frequency=100.0, inner_radius_proportion=0.7)
    jobs = {"a": ("am", ja, am.N), "g": ("g", jg, gl.N), "c": ("cyl", jc, cy.N)}
    alone = _run_alone(meshes, c, jobs, ["a", "g", "c"])

    b = Batch(1 << 16, 8)
    b.configure(chunk=10, occupancy=4, graph_chunks=2)
    sa, sg, sc = b.add_mesh(meshes["am"]), b.add_mesh(meshes["g"]), b.add_cyl(c)
    ida = b.submit(sa, **ja)
    b.advance(20)                     # job g arrives while a runs
    idg = b.submit(sg, **jg)
    b.advance(30)
    assert b.job_status(ida) == (50, True)
    b.retire(ida)
    b.compact()                       # a leaves; g keeps running from its slot
    idc = b.submit(sc, **jc)
    b.run()
    assert b.status() == 0
    got = {"g": (b.get(idg, gl.N), b.signal(idg, np.array([[1e-3, 2e-3, 0.5e-3]], F)), b.counts(idg)),
           "c": (b.get(idc, cy.N), b.signal(idc, np.array([[1e-3, 2e-3, 0.5e-3]], F)), b.counts(idc))}
    for name in ("g", "c"):
        (p1, m1, mo1, c1, f1), s1, n1 = alone[name]
        (p2, m2, mo2, c2, f2), s2, n2 = got[name]
        assert np.array_equal(p1.view(np.uint32), p2.view(np.uint32)), name
        assert np.array_equal(m1.view(np.uint32), m2.view(np.uint32)), name
        assert np.array_equal(mo1.view(np.uint32), mo2.view(np.uint32)), name
        assert np.array_equal(c1, c2) and np.array_equal(f1, f2), name
        assert np.array_equal(n1, n2), name
        assert np.allclose(s1, s2, rtol=1e-12, atol=1e-9), name
    info = b.info()
    assert info["graph_launches"] > 0 and info["jobs"] == 2
