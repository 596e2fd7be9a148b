#!/usr/bin/env python3
"""Generate the golden fixtures that pin the CPU oracle to the reference.

Runs the reference's own CPU code (compiled from its sources by
oracle/build_ref.py into oracle/_ref/) on seeded substrates written by
dsim_gb300.substrates, and stores inputs and outputs in tests/golden/*.npz:

  mesh_am.npz   closed tubes with axon + myelin membranes, permeable
  mesh_g.npz    closed tubes with glia membranes, permeable
  cyl.npz       packed parallel cylinders (dSim2), permeable, myelin layer

Each fixture holds the substrate text, the reference's parsed arrays and
grid, the initial state after resetSpins()/reset() (positions from rand(),
compartments from the reference's own assignment, MWC seeds), the per-step
draws that the reference's MWC generator produced (regenerated from the
seeds by the oracle's restatement of myRandn and checked against the
reference's final seeds), and the reference's state and signal after the
steps.  Also extracts the hand collision case of the reference's MATLAB test
dSim3/matlab_tests/run_tests/collisions01.m into matlab_collisions.json.

The sequencer fixtures hold the reference's own update(), computeTensor() and
results writer run on gradient tables: seq_*.npz from dSim3/src/diffusion.cpp
(refharness/seq3.cpp), seq2_*.npz from dSim2/src/diffusion.cpp
(refharness/seq2.cpp).

Run here (needs the reference tree):  python3 tests/golden/make_golden.py
[--only seq2]  (--only regenerates one group of fixtures)
"""
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import build_ref  # noqa: E402
import oracle as O  # noqa: E402
from dsim_gb300 import substrates as S  # noqa: E402

REFERENCE = build_ref.reference_dir()


def run(exe, **kw):
    args = [exe] + ["%s=%s" % (k, v) for k, v in kw.items()]
    p = subprocess.run(args, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("%s failed: %s" % (exe, p.stderr[-2000:]))
    return O.read_dump(kw["out"])


def mwc_draws(seed0, N, iters):
    seeds = seed0.reshape(-1, 2).copy()
    d = np.zeros((iters, N, 4), np.float32)
    for it in range(iters):
        for i in range(N):
            out, s = O.myrandn(seeds[i])
            d[it, i] = out
            seeds[i] = s
    return d, seeds.reshape(-1)


def mesh_fixture(name, membranes, perm, seed, harness, tmp):
    tube = S.beaded_tubes(n_axons=3, verts_per_ring=12, ring_spacing=1.0, length=16.0, box=12.0,
                          closed=True, membranes=membranes, seed=seed, allow_overlap=False,
                          bead_period=8.0)
    path = os.path.join(tmp, name + ".mesh")
    S.write_mesh_file(path, tube)
    N, iters, ss, dt = 400, 64, 10.0, 0.01
    params = dict(N=N, seed=seed, spaceScale=ss, dt=dt, extraAdc=2.0, myelinAdc=0.2, intraAdc=2.0,
                  perm=perm, extraT2=80.0, myelinT2=7.5, intraT2=60.0, startBox=0.9, gx=40.0,
                  gy=-20.0, gz=60.0, gamma=42576.0, iters=iters, reflType=1)
    r = run(harness, mesh=path, out=os.path.join(tmp, name + ".bin"), **params)
    draws, seeds_end = mwc_draws(r["seed0"], N, iters)
    assert np.array_equal(seeds_end, r["seed1"]), "MWC restatement disagrees with the reference"
    with open(path) as fh:
        text = fh.read()
    cc = r["cubeCounter"]
    maxtpc = int(r["grid"][2])
    dense = r["trianglesInCubes"].reshape(-1, maxtpc) if maxtpc else np.zeros((len(cc), 0), np.uint32)
    lists = np.concatenate([dense[c, :cc[c]] for c in range(len(cc))]) if cc.sum() else np.zeros(0, np.uint32)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), mesh_text=np.frombuffer(text.encode(), np.uint8),
                        params=json.dumps(params), counts=r["counts"], vertices=r["vertices"],
                        trgls=r["trgls"], triInfo=r["triInfo"], helpers=r["helpers"],
                        maxabs=r["maxabs"], grid=r["grid"], cubeLength=r["cubeLength"],
                        cubeCounter=cc, cellLists=lists.astype(np.uint32), stdDevs=r["stdDevs"],
                        T2=r["T2"], pos0=r["pos0"], seed0=r["seed0"], spins0=r["spins0"],
                        draws=draws, pos1=r["pos1"], seed1=r["seed1"], spins1=r["spins1"],
                        signal=r["signal"])
    return r


def cyl_fixture(name, harness, tmp):
    xy, rad = S.packed_cylinders(n=64, cell=19.0, fraction=0.5, seed=3)
    path = os.path.join(tmp, name + ".fibers")
    S.write_cylinder_file(path, xy, rad)
    N, iters = 400, 64
    params = dict(N=N, seed=3, spaceScale=10.0, dt=0.01, extraAdc=2.0, intraAdc=2.0, myelinAdc=0.2,
                  extraT2=80.0, intraT2=70.0, myelinT2=8.0, perm=0.05, inner=0.7, gx=80.0, gy=0.0,
                  gz=0.0, gamma=42576.0, iters=iters)
    r = run(harness, fibers=path, out=os.path.join(tmp, name + ".bin"), **params)
    seed0 = r["seed0"].reshape(-1, 4)[:, :2].reshape(-1).copy()
    draws, seeds_end = mwc_draws(seed0, N, iters)
    assert np.array_equal(seeds_end.reshape(-1, 2), r["seed1"].reshape(-1, 4)[:, :2])
    with open(path) as fh:
        text = fh.read()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), fibers_text=np.frombuffer(text.encode(), np.uint8),
                        params=json.dumps(params), fiberPos=r["fiberPos"], maxR=r["maxR"], grid=r["grid"],
                        cubeLength=r["cubeLength"], cubeCounter=r["cubeCounter"], cubes=r["cubes"],
                        pos0=r["pos0"], seed0=r["seed0"], params0=r["params0"], draws=draws,
                        pos1=r["pos1"], seed1=r["seed1"], params1=r["params1"], signal=r["signal"])
    return r


def matlab_collision_case():
    """Numbers of dSim3/matlab_tests/run_tests/collisions01.m:6-12."""
    path = os.path.join(REFERENCE, "dSim3", "matlab_tests", "run_tests", "collisions01.m")
    with open(path) as fh:
        text = fh.read()
    vals = {k: float(v) for k, v in re.findall(r"(\w+)\s*=\s*(-?[0-9.]+(?:e-?\d+)?)\s*;", text)}
    keys = ["oPosx", "oPosy", "oPosz", "posx", "posy", "posz", "x1", "y1", "z1", "x2", "y2", "z2",
            "x3", "y3", "z3", "intPx", "intPy", "intPz"]
    case = {k: vals[k] for k in keys}
    case["source"] = "dSim3/matlab_tests/run_tests/collisions01.m:6-12"
    with open(os.path.join(HERE, "matlab_collisions.json"), "w") as fh:
        json.dump(case, fh, indent=1)


SEQ_CONFIG = dict(numSpins=20000, gamma=42576.0, extraAdc=2.0, intraAdc=1.8, myelinAdc=0.2, spaceScale=25.0,
                  permeability=0.001, fiberFile="tubes.mesh")


def _tensor_signals(rows):
    """Per row and signal column (total, compartments 0-3): S0 exp(-b g^T D g)
    for five anisotropic tensors D (um^2/ms) and five S0."""
    rng = np.random.default_rng(17)
    out = np.zeros((len(rows), 5))
    for c in range(5):
        A = rng.normal(size=(3, 3))
        Q, _ = np.linalg.qr(A)
        D = Q @ np.diag(np.sort(rng.uniform(0.2, 2.5, 3))) @ Q.T
        s0 = rng.uniform(0.5, 1.0)
        for k, r in enumerate(rows):
            g = np.asarray(r[3:6], np.float64)
            n = np.linalg.norm(g)
            b = (2 * np.pi * 42576.0 * n * 1e-9 * r[0]) ** 2 * (r[1] - r[0] / 3.0)
            u = g / n if n > 0 else g
            out[k, c] = s0 * np.exp(-b * (u @ D @ u))
    return out


def seq_fixture(name, rows, timeStep, spu, seq, tmp):
    """The reference's update() / computeTensor() / writer on a gradient table
    (refharness/seq3.cpp): every updateSpins call with its gradient, the
    resets and reads, the results table, the fits and the results file."""
    rows = np.asarray(rows, np.float32).reshape(-1, 6)
    sig = _tensor_signals(rows)
    runs = O.sequencer_runs(rows, timeStep, spu)
    read = [k for k in range(len(rows)) if runs[k] is not None]
    g = os.path.join(tmp, name + ".g")
    sg = os.path.join(tmp, name + ".s")
    rows.tofile(g)
    given = np.zeros_like(sig)           # returned in read order; rows never read get none
    given[:len(read)] = sig[read]
    given.tofile(sg)
    outm = os.path.join(tmp, name + ".m")
    r = run(seq, grads=g, signals=sg, timeStep=timeStep, stepsPerUpdate=spu, outm=outm,
            out=os.path.join(tmp, name + ".bin"), **SEQ_CONFIG)
    with open(outm, "rb") as fh:
        mtext = fh.read()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), rows=rows, signals=sig, timeStep=np.float32(timeStep),
                        stepsPerUpdate=np.uint32(spu), config=json.dumps(SEQ_CONFIG), calls=r["calls"],
                        events=r["events"], results=r["results"], tensors=r["tensors"], eigenvecs=r["eigenvecs"],
                        lambdas=r["lambdas"], md=r["md"], fa=r["fa"], rd=r["rd"],
                        mfile=np.frombuffer(mtext, np.uint8))
    return r


def seq_fixtures(tmp):
    from dsim_gb300.engine import parse_grads
    from dsim_gb300.jobs import fibonacci_dirs, pgse_gmag
    seq = build_ref.sequencer_harness()
    # the reference's own gradient table
    seq_fixture("seq_simgrads", parse_grads(path=os.path.join(REFERENCE, "dSim3", "sim.grads")), 0.01, 10, seq, tmp)
    # Fibonacci directions at two b-values, with a row whose readout rounds to
    # zero updates (its signal is never read) in the middle
    rows = [[5.0, 20.0, 1.0, 0.0, 0.0, 0.0]]
    for b in (0.5, 1.0):
        for d in fibonacci_dirs(12):
            rows.append([5.0, 20.0, 1.0, *(pgse_gmag(b, 5.0, 20.0) * d)])
    rows.insert(7, [5.0, 20.0, 0.001, *(pgse_gmag(1.0, 5.0, 20.0) * fibonacci_dirs(12)[3])])
    seq_fixture("seq_fib", rows, 0.005, 1, seq, tmp)
    # six directions span five tensor components: the rank-deficient fit
    rows = [[8.0, 25.0, 2.0, 0.0, 0.0, 0.0]] + [[8.0, 25.0, 2.0, *(pgse_gmag(1.5, 8.0, 25.0) * d)]
                                               for d in fibonacci_dirs(6)]
    seq_fixture("seq_rank6", rows, 0.01, 5, seq, tmp)


SEQ2_CONFIG = dict(numSpins=999, spaceScale=50.0, radiusMean=1.5, spacingMean=0.3, crossFraction=0.1, useGpu=1,
                   fiberFile="sim.fibers")


def seq2_fixture(name, rows, timestep, iterations, seq, tmp):
    """The reference's dSim2 update() and results writer on a gradient table
    (refharness/seq2.cpp): every update call with its gradient, the resets and
    reads, and the results file (header, one block per run, timing)."""
    rows = np.asarray(rows, np.float32).reshape(-1, 6)
    sig = _tensor_signals(rows)[:, 0]
    runs = O.sequencer_runs(rows, timestep, iterations)
    read = [k for k in range(len(rows)) if runs[k] is not None]
    g = os.path.join(tmp, name + ".g")
    sg = os.path.join(tmp, name + ".s")
    rows.tofile(g)
    np.ascontiguousarray(sig[read], np.float64).tofile(sg)   # returned in read order
    outm = os.path.join(tmp, name + ".m")
    r = run(seq, grads=g, signals=sg, timestep=timestep, iterations=iterations, outm=outm,
            out=os.path.join(tmp, name + ".bin"), **SEQ2_CONFIG)
    with open(outm, "rb") as fh:
        mtext = fh.read()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), rows=rows, signals=sig, timeStep=np.float32(timestep),
                        stepsPerUpdate=np.uint32(iterations), config=json.dumps(SEQ2_CONFIG), calls=r["calls"],
                        events=r["events"], mfile=np.frombuffer(mtext, np.uint8))
    return r


def seq2_fixtures(tmp):
    from dsim_gb300.engine import parse_grads
    from dsim_gb300.jobs import fibonacci_dirs, pgse_gmag
    seq = build_ref.sequencer_harness(2)
    # the reference's own dSim2 gradient table
    seq2_fixture("seq2_simgrads", parse_grads(path=os.path.join(REFERENCE, "dSim2", "sim.grads")), 0.005, 10, seq,
                 tmp)
    # Fibonacci directions, a b = 0 row, and a row whose readout rounds to
    # zero updates (its signal is never read)
    rows = [[6.0, 15.0, 1.5, 0.0, 0.0, 0.0]] + [[6.0, 15.0, 1.5, *(pgse_gmag(1.0, 6.0, 15.0) * d)]
                                               for d in fibonacci_dirs(9)]
    rows.insert(4, [6.0, 15.0, 0.001, *(pgse_gmag(0.5, 6.0, 15.0) * fibonacci_dirs(9)[2])])
    seq2_fixture("seq2_fib", rows, 0.01, 3, seq, tmp)


def main():
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", choices=["seq2"], default=None)
    args = ap.parse_args()
    if REFERENCE is None:
        raise SystemExit("the reference tree is not present (set DSIM_REFERENCE)")
    h3, h2 = build_ref.build(REFERENCE)
    with tempfile.TemporaryDirectory() as tmp:
        if args.only is None:
            mesh_fixture("mesh_am", "AM", 0.05, 11, h3, tmp)
            mesh_fixture("mesh_g", "G", 0.2, 12, h3, tmp)
            cyl_fixture("cyl", h2, tmp)
            seq_fixtures(tmp)
        seq2_fixtures(tmp)
    if args.only is None:
        matlab_collision_case()
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
