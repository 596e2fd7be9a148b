"""The serving form (include/dsim_serve.h): jobs submitted while others run
are admitted as slots free up, their work shares the step launches, and each
job's signals equal the job run alone (FP64 sums over the same per-spin
states, added in another order: relative 1e-12).  Also the autotuner: it
restores the batch state it timed on, so results after tuning equal results
without it."""
import time

import numpy as np
import pytest

from scenarios import CylCase, MeshCase

pytestmark = pytest.mark.gpu
F = np.float32


def _jobs(tmp_path):
    am = MeshCase(tmp_path, membranes="AM", permeability=0.05, N=900)
    gl = MeshCase(tmp_path, membranes="G", permeability=0.1, N=1300, seed=4)
    cy = CylCase(tmp_path, permeability=0.02, inner=0.7, N=800)
    ss = F(cy.spaceScale)
    csd = [float(np.sqrt(F(2) * (F(adc) / (ss * ss)) * F(cy.dt))) for adc in (2.0, 0.2, 2.0)] + [0.0]
    grads = np.array([[1e-3, 0, 0], [0, 2e-3, 0], [0.5e-3, 0.5e-3, 1e-3]], F)
    jobs = []
    for k in range(6):
        if k % 3 == 0:
            c, sub = am, "am"
        elif k % 3 == 1:
            c, sub = gl, "g"
        else:
            c, sub = cy, "cyl"
        if sub == "cyl":
            kw = dict(pos=c.pos, comp=np.full(c.N, 2, np.uint8), fiber=None, steps=30 + 10 * k, dt=c.dt,
                      step_sd=csd, T2=[70.0, 8.0, 80.0, 0.0], phase_constant=c.pc, seed=100 + k,
                      permeability=0.02, waveform="pgse", delta=0.1, Delta=0.2, inner_radius_proportion=0.7)
        else:
            kw = dict(pos=c.pos, comp=c.comp, fiber=c.fiber.astype(np.uint32), steps=30 + 10 * k, dt=c.dt,
                      step_sd=c.stdDevs, T2=c.T2, phase_constant=c.pc, seed=100 + k,
                      permeability=c.permeability, waveform="ogse" if k == 3 else "pgse", delta=0.1,
                      Delta=0.2, frequency=200.0)
        jobs.append((sub, kw, c.N))
    return am, gl, cy, jobs, grads


def _alone(meshes, cyl, sub, kw, grads):
    from dsim_gb300.engine import Batch
    b = Batch(1 << 14, 2)
    b.configure(chunk=10, occupancy=4, graph_chunks=2)
    sid = b.add_cyl(cyl) if sub == "cyl" else b.add_mesh(meshes[sub])
    j = b.submit(sid, **kw)
    b.run()
    out = b.signal(j, grads)
    b.close()
    return out


def test_served_jobs_equal_alone(engine, tmp_path):
    from dsim_gb300.engine import Cylinders, Mesh, Server
    am, gl, cy, jobs, grads = _jobs(tmp_path)
    meshes = {"am": Mesh.load(am.path, am.spaceScale), "g": Mesh.load(gl.path, gl.spaceScale)}
    c = Cylinders.load(cy.path, cy.spaceScale)
    want = [_alone(meshes, c, sub, kw, grads) for sub, kw, _ in jobs]

    # arena of 3 jobs' worth of slots: later arrivals wait for slots to free up
    srv = Server(spin_capacity=4096, job_capacity=3, hbm_cap=64e9)
    sids = {"am": srv.add_mesh(meshes["am"]), "g": srv.add_mesh(meshes["g"]), "cyl": srv.add_cyl(c)}
    srv.configure(chunk=10, occupancy=4, graph_chunks=2)
    srv.start()
    tickets = []
    for k, (sub, kw, n) in enumerate(jobs):
        kw = dict(kw)
        pos, comp, fib = kw.pop("pos"), kw.pop("comp"), kw.pop("fiber")
        tickets.append(srv.submit(sids[sub], pos, comp, fib, grads, **kw))
        time.sleep(0.002 * (k % 2))
    srv.drain()
    st = srv.stats()
    srv.stop()
    assert st["errors"] == 0 and st["jobs_done"] == len(jobs)
    assert st["max_inflight"] >= 2
    admits = []
    for t, w in zip(tickets, want):
        done, sig, times = srv.poll(t)
        assert done
        assert times[0] <= times[1] <= times[2]
        admits.append(times[1])
        assert np.allclose(sig, w, rtol=1e-12, atol=1e-9)
    # with 3 job slots the later jobs were admitted only after earlier ones left
    assert max(admits) > min(admits)
    srv.close()


def test_autotune_restores_state(engine, tmp_path):
    from dsim_gb300.engine import Batch, Mesh
    am = MeshCase(tmp_path, membranes="AM", permeability=0.05, N=1500)
    m = Mesh.load(am.path, am.spaceScale)
    kw = dict(pos=am.pos, comp=am.comp, fiber=am.fiber.astype(np.uint32), steps=60, dt=am.dt,
              step_sd=am.stdDevs, T2=am.T2, phase_constant=am.pc, seed=9, permeability=am.permeability,
              waveform="pgse", delta=0.2, Delta=0.3)
    ref = Batch(1 << 14, 2)
    sid = ref.add_mesh(m)
    j = ref.submit(sid, **kw)
    ref.run()
    want = ref.get(j, am.N)
    ref.close()
    b = Batch(1 << 14, 2)
    sid = b.add_mesh(m)
    j = b.submit(sid, **kw)
    best, ms = b.autotune(trial_steps=20)
    assert best["occupancy"] in (4, 5, 6, 8) and best["chunk"] in (20, 40, 100, 200, 500, 1000) and ms > 0
    assert best["fine_per_ref"] in (1.0, 1.5, 2.0, 2.5) and best["block"] in (64, 128, 256)
    assert b.job_status(j) == (0, False)
    b.run()
    got = b.get(j, am.N)
    for a, w in zip(got, want):
        assert np.array_equal(np.asarray(a).view(np.uint8), np.asarray(w).view(np.uint8))
    b.close()


def test_admission_counts_the_precision_forms_device_memory(engine, tmp_path):
    """The HBM cap counts, from the first job of a precision form on, the
    arena's FP64 fields (64 B per spin slot) and that mesh's FP64 triangle
    table (128 B per triangle): a cell-local job that can never fit under the
    cap with them is refused at submission (instead of waiting forever), the
    same job in the plain form is served, and the peak admitted bytes of a
    served cell-local job include them."""
    from dsim_gb300.engine import Mesh, Server
    am, gl, cy, jobs, grads = _jobs(tmp_path)
    m = Mesh.load(am.path, am.spaceScale)
    sub, kw, n = jobs[0]
    kw = dict(kw)
    pos, comp, fib = kw.pop("pos"), kw.pop("comp"), kw.pop("fiber")
    cap_slots = 1 << 14
    probe = Server(spin_capacity=cap_slots, job_capacity=2, hbm_cap=64e9)
    sid = probe.add_mesh(m)
    probe.configure(chunk=10, occupancy=4, graph_chunks=2)
    probe.start()
    t = probe.submit(sid, pos, comp, fib, grads, **kw)
    probe.drain()
    plain_peak = probe.stats()["hbm_peak"]
    probe.stop()
    probe.close()
    # a cap just above the plain job's peak: the plain job is served, the cell-local one refused
    srv = Server(spin_capacity=cap_slots, job_capacity=2, hbm_cap=plain_peak + 1024)
    sid = srv.add_mesh(m)
    srv.configure(chunk=10, occupancy=4, graph_chunks=2)
    srv.start()
    with pytest.raises(Exception):
        srv.submit(sid, pos, comp, fib, grads, local=True, **kw)
    t = srv.submit(sid, pos, comp, fib, grads, **kw)
    srv.drain()
    assert srv.poll(t)[0] and srv.stats()["errors"] == 0
    srv.stop()
    srv.close()
    # with room, the cell-local job's peak includes the arena's FP64 fields
    srv = Server(spin_capacity=cap_slots, job_capacity=2, hbm_cap=64e9)
    sid = srv.add_mesh(m)
    srv.configure(chunk=10, occupancy=4, graph_chunks=2)
    srv.start()
    t = srv.submit(sid, pos, comp, fib, grads, local=True, **kw)
    srv.drain()
    assert srv.poll(t)[0]
    assert srv.stats()["hbm_peak"] >= plain_peak + cap_slots * 64
    srv.stop()
    srv.close()
