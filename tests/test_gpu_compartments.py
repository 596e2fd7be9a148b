"""GPU compartment assignment against the reference's findSpinsInFibers.

The golden fixtures hold the reference's own assignment (compartment and
fiber per spin after resetSpins, dSim3/src/spinSystem.cpp:1386-1407 and
1615-1852) for two closed-tube meshes; the kernel must reproduce it for the
same positions.  On a larger closed mesh the assignment must agree with the
tube geometry wherever the geometry is unambiguous."""
import json
import os

import numpy as np
import pytest

import oracle as O
from scenarios import MeshCase

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name", ["mesh_am", "mesh_g"])
def test_compartments_match_reference(engine, tmp_path, name):
    from dsim_gb300.engine import Mesh, Spins
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    prm = json.loads(str(g["params"]))
    path = tmp_path / "mesh.txt"
    path.write_bytes(g["mesh_text"].tobytes())
    m = Mesh.load(str(path), prm["spaceScale"])
    _, _, comp0, fib0 = O.spin_fields(g["spins0"])
    N = len(comp0)
    s = Spins(N)
    s.set(g["pos0"], np.ones(N, np.float32), np.zeros(N, np.float32), np.zeros(N, np.uint8),
          np.full(N, 0xFFFF, np.uint16))
    moved = m.compartments(s, seed=3)
    pos, _, _, comp, fib = s.get()
    assert s.status() == 0 and moved == 0
    assert np.array_equal(pos.view(np.uint32), g["pos0"].view(np.uint32))
    assert np.array_equal(comp, comp0)
    assert np.array_equal(fib, fib0)
    assert len(np.unique(comp0)) >= 2


@pytest.mark.parametrize("membranes", ["AM", "G"])
def test_compartments_follow_tube_geometry(engine, tmp_path, membranes):
    from dsim_gb300.engine import Mesh, Spins
    case = MeshCase(tmp_path, membranes=membranes, N=20000, seed=7)
    m = Mesh.load(case.path, case.spaceScale)
    s = Spins(case.N)
    s.set(case.pos, case.mag, case.phase, np.zeros(case.N, np.uint8), np.full(case.N, 0xFFFF, np.uint16))
    m.compartments(s, seed=5)
    assert s.status() == 0
    pos, _, _, comp, fib = s.get()
    um = pos.reshape(-1, 3).astype(np.float64) * case.spaceScale
    inner = 1 if membranes == "AM" else 3
    checked = 0
    for i, ((cx, cy), r0) in enumerate(zip(case.tube["centres"], case.tube["radii"])):
        r = r0 * (1 + 0.2 * np.sin(2 * np.pi * um[:, 2] / 8.0))
        d = np.hypot(um[:, 0] - cx, um[:, 1] - cy)
        core = (d < 0.85 * r) & (np.abs(um[:, 2]) < 7.5)
        assert np.all(comp[core] == inner) and np.all(fib[core] == i)
        checked += core.sum()
        if membranes == "AM":
            shell = (d > 1.08 * r) & (d < 1.17 * r) & (np.abs(um[:, 2]) < 7.5)
            assert np.all(comp[shell] == 2) and np.all(fib[shell] == i)
    far = np.ones(case.N, bool)
    for (cx, cy), r0 in zip(case.tube["centres"], case.tube["radii"]):
        far &= np.hypot(um[:, 0] - cx, um[:, 1] - cy) > 1.25 * 1.2 * r0 * 1.05
    assert np.all(comp[far] == 0) and np.all(fib[far] == 0xFFFF)
    assert checked > 100 and far.sum() > 100
