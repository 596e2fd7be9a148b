"""The simulate call's host parts (include/dsim_sim.h), no GPU needed:
config dialects, gradient files, the PGSE sequencer against a state-machine
replay of the reference's update(), and the tensor fit against a numpy
restatement of computeTensor."""
import numpy as np
import pytest

import oracle as O

CFG3 = """
// dSim3-style keys
app: {
    stepsPerUpdate = 5;   # five steps per update
    useGpu = true;
    useDisplay = false;
    writeOut = true;
};
sim: {
    numSpins = 2048;
    gyroMagneticRatio = 42576.0;
    timeStep = 0.004;
    extraAdc = 1.9; intraAdc = 1.7; myelinAdc = 0.2;
    extraT2 = 70.0; intraT2 = 60.0; myelinT2 = 9.0;
    permeability = 0.001;
    spaceScale = 12.5;
    startBox = 0.8;
    gradsFile = "run.grads";
    outFile = "out.m";
};
/* fibers */
fibers: { fiberFile = "tubes.txt"; };
"""

CFG2 = """
app: { useGpu = false; useDisplay = true; stepsPerUpdate = 8; };
sim: {
    numSpins = 999;
    gyromagneticRatio = 42576.0;
    timestep = 0.01;
    extraAdc = 2.0; intraAdc = 2.0; myelinAdc = 0.1;
    spaceScale = 10.0;
    permeability = -3.0;
    gradsStr = "12.0 20.0 1.0 40.0 0.0 0.0";
};
fibers: { file = "cyl.fibers"; innerRadiusFraction = 0.6; radiusMean = 0.75; };
"""


@pytest.fixture(scope="module")
def lib():
    from dsim_gb300 import build
    build.build()


def test_config_dialects(lib, tmp_path):
    from dsim_gb300.engine import load_config
    p3 = tmp_path / "a.cfg"
    p3.write_text(CFG3)
    c = load_config(p3)
    assert c["dialect"] == 3 and c["stepsPerUpdate"] == 5 and c["numSpins"] == 2048
    assert c["useGpu"] == 1 and c["useDisplay"] == 0 and c["writeOut"] == 1
    assert np.float32(c["timeStep"]) == np.float32(0.004) and np.float32(c["spaceScale"]) == np.float32(12.5)
    assert c["gradsFile"] == "run.grads" and c["outFile"] == "out.m" and c["fiberFile"] == "tubes.txt"
    assert np.float32(c["permeability"]) == np.float32(0.001) and np.float32(c["startBox"]) == np.float32(0.8)
    p2 = tmp_path / "b.cfg"
    p2.write_text(CFG2)
    c = load_config(p2)
    assert c["dialect"] == 2 and c["stepsPerUpdate"] == 8 and c["numSpins"] == 999
    assert np.isclose(c["permeability"], 1e-3) and np.float32(c["timeStep"]) == np.float32(0.01)
    assert c["fiberFile"] == "cyl.fibers" and c["gradsStr"].startswith("12.0 20.0")
    assert np.float32(c["innerRadiusFraction"]) == np.float32(0.6)
    bad = tmp_path / "bad.cfg"
    bad.write_text("sim: { numSpins = ; };")
    from dsim_gb300._lib import DsimError
    with pytest.raises(DsimError):
        load_config(bad)


def test_grads_rows_read_six_numbers_at_a_time(lib, tmp_path):
    from dsim_gb300.engine import parse_grads
    p = tmp_path / "g.grads"
    p.write_text("10.00 12.0669 1.00 0.0 0.0 0.0\n\n10 12.0669 1\n80 80 0\n5 6 7\n")
    rows = parse_grads(path=p)
    assert rows.shape == (2, 6)
    assert np.array_equal(rows[1], np.float32([10, 12.0669, 1, 80, 80, 0]))
    assert parse_grads(text="1 2 3 4 5 6 7 8 9 10 11 12").shape == (2, 6)
    from dsim_gb300._lib import DsimError
    with pytest.raises(DsimError):
        parse_grads(text="1 2 x 4 5 6")


@pytest.mark.parametrize("spu,dt", [(10, 0.005), (7, 0.004), (1, 0.01)])
def test_sequencer_matches_reference_update(lib, spu, dt):
    from dsim_gb300.engine import pgse_schedule
    rows = np.float32([[10.0, 12.0669, 1.0, 0.0, 0.0, 0.0], [10.0, 12.0669, 1.0, 80.0, 80.0, 0.0],
                       [3.0, 3.0, 0.5, 0.0, -20.0, 5.0], [0.0, 8.0, 0.0, 1.0, 2.0, 3.0],
                       [18.0, 19.31, 1.0, 51.0, 0.0, 0.0]])
    runs = O.sequencer_runs(rows, dt, spu)
    assert len(runs) == len(rows)
    from dsim_gb300._lib import DsimError
    for row, want in zip(rows, runs):
        if want is None:
            # the reference never reads this row's signal (readout of zero updates)
            with pytest.raises(DsimError):
                pgse_schedule(row, dt, spu)
            continue
        got = pgse_schedule(row, dt, spu)
        assert np.array_equal(got, np.repeat(want, spu, axis=0)), row
    assert sum(w is None for w in runs) == 1


def test_tensor_fit_matches_reference_fit(lib):
    from dsim_gb300.engine import tensor_fit
    from dsim_gb300.jobs import fibonacci_dirs, pgse_gmag
    rng = np.random.default_rng(4)
    Q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
    Dt = Q @ np.diag([2.0e-3 * 1e3, 0.6, 0.3]) @ Q.T * 1e-0   # um^2/ms
    delta, Delta = 10.0, 30.0
    rows = [[delta, Delta, 1.0, 0, 0, 0]]
    for b in (1.0, 2.0):
        G = pgse_gmag(b, delta, Delta)
        for d in fibonacci_dirs(12):
            rows.append([delta, Delta, 1.0, *(G * d)])
    rows = np.float32(rows)
    # signals as the reference would measure them for diffusion tensor Dt
    g = rows[:, 3:6].astype(np.float64)
    n = np.linalg.norm(g, axis=1)
    bv = ((2.0 * 3.1415926535 * 42576.0) * n / 1e9 * rows[:, 0]) ** 2 * (rows[:, 1] - rows[:, 0] / 3.0)
    u = np.where(n[:, None] > 0, g / np.where(n > 0, n, 1)[:, None], 0)
    S = np.exp(-bv * np.einsum("ij,jk,ik->i", u, Dt, u))
    got = tensor_fit(rows, S)
    D, lam, md, fa, rd = O.tensor_fit_reference(rows, S)
    assert np.allclose(got["tensor"], D, rtol=1e-4, atol=1e-6)
    assert np.allclose(got["tensor"], Dt, rtol=1e-3, atol=1e-5)
    assert np.allclose(got["eigvals"], lam, rtol=1e-4)
    assert np.isclose(got["md"], md, rtol=1e-4) and np.isclose(got["fa"], fa, rtol=1e-4)
    assert np.isclose(got["rd"], rd, rtol=1e-4)
    V = got["eigvecs"]
    assert np.allclose(V.T @ V, np.eye(3), atol=1e-9)
    assert np.allclose(got["tensor"] @ V, V * got["eigvals"].astype(np.float64)[None, :], atol=1e-6)


def test_tensor_fit_rank_deficient_table_is_minimum_norm(lib):
    """Six Fibonacci directions span only five tensor components: the fit must
    stay finite and agree with the reference's pseudo-inverse solution."""
    from dsim_gb300.engine import tensor_fit
    from dsim_gb300.jobs import fibonacci_dirs, pgse_gmag
    delta, Delta = 5.0, 20.0
    rows = [[delta, Delta, 1.0, 0, 0, 0]] + [[delta, Delta, 1.0, *(pgse_gmag(1.0, delta, Delta) * d)]
                                            for d in fibonacci_dirs(6)]
    rows = np.float32(rows)
    S = np.array([1.0] + [np.exp(-2.0)] * 6)
    got = tensor_fit(rows, S)
    D, lam, md, fa, rd = O.tensor_fit_reference(rows, S)
    assert np.all(np.isfinite(got["tensor"]))
    assert np.allclose(got["tensor"], D, rtol=1e-4, atol=1e-5)
