"""The simulate call end to end on the GPU (include/dsim_sim.h): a sim.cfg
names the fiber file and the gradient table; the sequencer walks every
gradient, the tensor fit and the results file follow.  With the membranes
far from the spins the signals must follow free diffusion exp(-bD) (in the
exact form of the walk's time steps, from the sequencer's own gradient
schedule) within 3 standard errors and no other slack, and the fitted mean
diffusivity must equal D."""
import numpy as np
import pytest

from scenarios import CylCase

pytestmark = pytest.mark.gpu

N_SPINS = 100_000


def _far_tube_mesh(path):
    from dsim_gb300 import substrates as S
    V, T = S.tube_mesh(45.0, 45.0, lambda z: np.full_like(z, 0.8), -5.0, 5.0, 1.0, 8, closed=True)
    S.write_mesh_file(str(path), {"vertices": V, "trgls": T, "membrane": np.full(len(T), 2),
                                  "fiber": np.zeros(len(T), int)})


def test_simulate_free_diffusion_mesh(engine, tmp_path):
    from dsim_gb300.engine import grad_scaled, pgse_schedule, phase_constant, simulate, std_devs, tensor_fit
    from dsim_gb300.jobs import fibonacci_dirs, pgse_gmag
    from test_gpu_physics import discrete_free_signal, free_se
    _far_tube_mesh(tmp_path / "far.txt")
    delta, Delta, D = 5.0, 20.0, 2.0
    rows = [[delta, Delta, 1.0, 0.0, 0.0, 0.0]]
    for b in (0.5, 1.0):
        for d in fibonacci_dirs(12):
            rows.append([delta, Delta, 1.0, *(pgse_gmag(b, delta, Delta) * d)])
    np.savetxt(tmp_path / "run.grads", np.array(rows), fmt="%.6f")
    (tmp_path / "sim.cfg").write_text(
        'app: { stepsPerUpdate = 10; writeOut = true; };\n'
        'sim: { numSpins = %d; gyroMagneticRatio = 42576.0; timeStep = 0.01; extraAdc = %g; intraAdc = %g;\n'
        '       myelinAdc = 0.1; extraT2 = 80.0; intraT2 = 80.0; myelinT2 = 7.5; permeability = 0.0;\n'
        '       spaceScale = 50.0; startBox = 0.2; gradsFile = "run.grads"; outFile = "%s"; };\n'
        'fibers: { fiberFile = "far.txt"; };\n' % (N_SPINS, D, D, tmp_path / "out.m"))
    sig, sec = simulate(tmp_path / "sim.cfg", seed=3, write_out=True)
    assert sig.shape == (len(rows), 5) and sec > 0
    bvals = np.array([0.0] + [0.5] * 12 + [1.0] * 12)
    t2 = np.exp(-(delta + Delta + 1.0) / 80.0)       # every run decays by T2 over delta + Delta + readout
    assert abs(sig[0, 0] - t2) < 1e-3
    dt, ss = 0.01, 50.0
    sd = std_devs(D, D, 0.1, ss, dt)[0]
    pc = phase_constant(42576.0, dt)
    want = np.array([discrete_free_signal(grad_scaled(pgse_schedule(r, dt, 10), ss), sd, pc) for r in rows])
    assert np.allclose(want, np.exp(-bvals * D), atol=5e-3)      # the continuous closed form
    se = free_se(want, N_SPINS)
    assert np.all(np.abs(sig[:, 0] / sig[0, 0] - want) <= 3 * se), (sig[:, 0] / sig[0, 0], want, se)
    assert np.allclose(sig[:, 1], sig[:, 0])        # every spin outside the tube (compartment 0)
    fit = tensor_fit(np.array(rows, np.float32), sig[:, 0])
    assert abs(fit["md"] - D) < 0.05 * D and fit["fa"] < 0.1
    text = (tmp_path / "out.m").read_text()
    assert text.count("mrSigTotal{m}(s)") == len(rows) and "md{m}(1)" in text and "tensor{m}{1}" in text
    # one shared walk for the whole table: same physics
    sig2, _ = simulate(tmp_path / "sim.cfg", seed=4, shared_walk=True)
    assert np.all(np.abs(sig2[:, 0] / sig2[0, 0] - want) <= 3 * se), (sig2[:, 0] / sig2[0, 0], want, se)


def test_simulate_cylinders_dsim2_config(engine, tmp_path):
    from dsim_gb300.engine import simulate
    case = CylCase(tmp_path, N=100)
    (tmp_path / "sim2.cfg").write_text(
        'app: { stepsPerUpdate = 10; };\n'
        'sim: { numSpins = 8000; gyromagneticRatio = 42576.0; timestep = 0.01; extraAdc = 2.0; intraAdc = 2.0;\n'
        '       myelinAdc = 0.2; spaceScale = 10.0; permeability = -9.0;\n'
        '       gradsStr = "10.0 20.0 1.0 0.0 0.0 0.0  10.0 20.0 1.0 60.0 0.0 0.0  10.0 20.0 1.0 0.0 0.0 60.0"; };\n'
        'fibers: { file = "%s"; innerRadiusFraction = 0.7; };\n' % case.path)
    sig, _ = simulate(tmp_path / "sim2.cfg", seed=2)
    assert sig.shape == (3, 5)
    assert 0.5 < sig[0, 0] <= 1.0                    # T2 decay only
    # restricted across the z-cylinders: less attenuation across (x) than along (z)
    assert 0 < sig[2, 0] < sig[1, 0] < sig[0, 0]
    sig2, _ = simulate(tmp_path / "sim2.cfg", seed=2, shared_walk=True)
    assert 0 < sig2[2, 0] < sig2[1, 0] < sig2[0, 0]
