"""The sequencer, the tensor fit and the results writer against the
reference's own code: update(), computeTensor() and the results writer of
dSim3/src/diffusion.cpp, run unchanged by oracle/refharness/seq3.cpp on three
gradient tables (the reference's own sim.grads; Fibonacci directions at two
b-values with a row whose readout rounds to zero updates; six directions,
which span only five tensor components).  The fixtures tests/golden/seq_*.npz
hold every updateSpins call with its gradient, the resets and reads, the
results table, the fits and the results file; tests/golden/make_golden.py
wrote them.

* dsim_pgse_schedule gives each row the gradient of every step of the
  reference's run, from the reset to the read, and refuses the row the
  reference never reads;
* dsim_tensor_fit equals computeTensor (JAMA SVD with its 1e-6 roundings,
  JAMA eigen-decomposition) within 1e-4;
* dsim_write_results writes the reference's results file: every line equal,
  the fitted numbers within 1e-4 (eigenvector columns up to sign).

The same for dSim2 (dSim2/src/diffusion.cpp:183-287 and its results header
1756-1770, run unchanged by oracle/refharness/seq2.cpp; fixtures
tests/golden/seq2_*.npz): the schedule of every run, and the results file line
for line (date and timing values aside).
"""
import json
import os
import re

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = ["seq_simgrads", "seq_fib", "seq_rank6"]
FIT_LINES = ("tensor{", "eigenvecs{", "eigenvals{", "md{", "fa{", "rd{")


def _load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def _walks(g):
    """Per row that the reference reads: its updateSpins calls from the reset
    to the read (each reset starts the next row)."""
    calls = g["calls"].reshape(-1, 7)
    out, last, nreset = {}, None, 0
    for kind, at in g["events"].reshape(-1, 2):
        if kind == 1:
            last = (nreset, int(at))
            nreset += 1
        else:
            row, r0 = last
            out[row] = calls[r0:int(at)]
    assert nreset == len(g["rows"])
    return out


@pytest.mark.parametrize("name", FIXTURES)
def test_schedule_equals_the_reference_sequencer(name):
    from dsim_gb300.engine import pgse_schedule
    g = _load(name)
    dt, spu = float(g["timeStep"]), int(g["stepsPerUpdate"])
    walks = _walks(g)
    for k, row in enumerate(g["rows"]):
        if k not in walks:
            with pytest.raises(Exception):
                pgse_schedule(row, dt, spu)
            continue
        w = walks[k]
        assert np.all(w[:, 6] == spu) and np.all(w[:, 5] == np.float32(dt))
        want = np.repeat(w[:, 2:5], spu, axis=0)
        got = pgse_schedule(row, dt, spu)
        assert got.shape == want.shape, (k, got.shape, want.shape)
        assert np.array_equal(got, want), k          # -0 and +0 compare equal
    # the results table: the row parameters as read, the signal of each read row
    res = g["results"].reshape(len(g["rows"]), 11)
    assert np.array_equal(res[:, :6], g["rows"])
    read = sorted(walks)
    assert np.array_equal(res[read, 6:11], g["signals"][read].astype(np.float32))
    assert not res[[k for k in range(len(res)) if k not in walks], 6:].any()


@pytest.mark.parametrize("name", FIXTURES)
def test_tensor_fit_equals_compute_tensor(name):
    from dsim_gb300.engine import tensor_fit
    g = _load(name)
    res = g["results"].reshape(len(g["rows"]), 11)
    T, E = g["tensors"].reshape(5, 3, 3), g["eigenvecs"].reshape(5, 3, 3)
    lam = g["lambdas"].reshape(5, 3)
    for c in range(5):
        f = tensor_fit(res[:, :6], res[:, 6 + c].astype(np.float64))
        assert np.allclose(f["tensor"], T[c], rtol=1e-4, atol=1e-6), (c, f["tensor"], T[c])
        assert np.allclose(f["eigvals"], lam[c], rtol=1e-4, atol=1e-6), (c, f["eigvals"], lam[c])
        for k in range(3):
            assert abs(abs(f["eigvecs"][:, k] @ E[c][:, k]) - 1.0) < 1e-4, (c, k)
        for key in ("md", "fa", "rd"):
            assert np.isclose(f[key], g[key][c], rtol=1e-4, atol=1e-6), (c, key, f[key], g[key][c])


def _numbers(line):
    return np.array([float(x) for x in re.findall(r"-?\d+\.?\d*(?:e[-+]?\d+)?", line.split("=", 1)[1])])


@pytest.mark.parametrize("name", FIXTURES)
def test_results_file_equals_the_reference_writer(name, tmp_path):
    from dsim_gb300.engine import write_results
    g = _load(name)
    cfg = json.loads(str(g["config"]))
    cfg.update(dialect=3, stepsPerUpdate=int(g["stepsPerUpdate"]), timeStep=float(g["timeStep"]), writeOut=1,
               useGpu=1)
    res = g["results"].reshape(len(g["rows"]), 11)
    out = tmp_path / "results.m"
    write_results(out, cfg, res[:, :6], res[:, 6:11].astype(np.float64))
    ours = out.read_text().split("\n")
    ref = g["mfile"].tobytes().decode().split("\n")
    assert len(ours) == len(ref)
    for a, b in zip(ours, ref):
        if a.startswith("% * * *") and b.startswith("% * * *"):
            continue                                   # the date of the run
        if a.startswith(FIT_LINES):
            assert a.split("=")[0] == b.split("=")[0]
            x, y = _numbers(a), _numbers(b)
            if a.startswith("eigenvecs{"):
                x, y = np.abs(x), np.abs(y)           # columns up to sign
            assert np.allclose(x, y, rtol=1e-4, atol=2e-6), (a, b)
        else:
            assert a == b, (a, b)


# ---- dSim2: update() and the results file of dSim2/src/diffusion.cpp -------
# (oracle/refharness/seq2.cpp: the reference's update() and results header,
# unchanged, on the gradient tables of tests/golden/seq2_*.npz: dSim2's own
# sim.grads, and Fibonacci directions with a row whose readout rounds to zero
# updates)
FIXTURES2 = ["seq2_simgrads", "seq2_fib"]


@pytest.mark.parametrize("name", FIXTURES2)
def test_dsim2_schedule_equals_the_reference_update(name):
    from dsim_gb300.engine import pgse_schedule
    g = _load(name)
    dt, its = float(g["timeStep"]), int(g["stepsPerUpdate"])
    walks = _walks(g)
    assert len(walks) < len(g["rows"]) or name == "seq2_simgrads"
    for k, row in enumerate(g["rows"]):
        if k not in walks:
            with pytest.raises(Exception):
                pgse_schedule(row, dt, its)
            continue
        w = walks[k]
        assert np.all(w[:, 6] == its) and np.all(w[:, 5] == np.float32(dt))
        got = pgse_schedule(row, dt, its)
        assert np.array_equal(got, np.repeat(w[:, 2:5], its, axis=0)), k


@pytest.mark.parametrize("name", FIXTURES2)
def test_dsim2_results_file_equals_the_reference_writer(name, tmp_path):
    from dsim_gb300.engine import write_results
    g = _load(name)
    c = json.loads(str(g["config"]))
    cfg = dict(dialect=2, stepsPerUpdate=int(g["stepsPerUpdate"]), timeStep=float(g["timeStep"]),
               numSpins=c["numSpins"], spaceScale=c["spaceScale"], fiberRadius=c["radiusMean"],
               fiberSpace=c["spacingMean"], crossFraction=c["crossFraction"], useGpu=c["useGpu"],
               fiberFile=c["fiberFile"])
    sig = np.zeros((len(g["rows"]), 5))
    sig[:, 0] = g["signals"]
    sig[[k for k in range(len(sig)) if k not in _walks(g)], 0] = np.nan   # as dsim_simulate reports them
    out = tmp_path / "results.m"
    write_results(out, cfg, g["rows"], sig, seconds=1.0)
    ours = out.read_text().split("\n")
    ref = g["mfile"].tobytes().decode().split("\n")
    assert len(ours) == len(ref), (len(ours), len(ref))
    for a, b in zip(ours, ref):
        if a.startswith("% * * *") and b.startswith("% * * *"):
            continue                                   # the date of the run
        if a.startswith(("stepsPerSec(m)", "totalTime(m)")):
            assert a.split("=")[0] == b.split("=")[0]  # the run's timing
            continue
        assert a == b, (a, b)
