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

Run here (needs the reference tree):  python3 tests/golden/make_golden.py
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


def main():
    if REFERENCE is None:
        raise SystemExit("the reference tree is not present (set DSIM_REFERENCE)")
    h3, h2 = build_ref.build(REFERENCE)
    with tempfile.TemporaryDirectory() as tmp:
        mesh_fixture("mesh_am", "AM", 0.05, 11, h3, tmp)
        mesh_fixture("mesh_g", "G", 0.2, 12, h3, tmp)
        cyl_fixture("cyl", h2, tmp)
    matlab_collision_case()
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
