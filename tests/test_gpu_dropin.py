"""The drop-in test: the reference's own host code on this project's GPU
libraries.

oracle/build_ref.py compiles the reference's SpinSystem (dSim3/src/spinSystem.cpp,
dSim2/src/spinSystem.cpp, from scratch copies prepared where the reference
tree exists) with useGpu = true and links it against libdsim3.so / libdsim2.so
instead of the reference's spinSystem.cu (oracle/refharness/dropin{3,2}.cpp).
The reference's own calls then allocate, copy and bind every device array and
set every constant through the C-ABI, and updateSpins / update take its GPU
branch (dSim3/src/spinSystem.cpp:1942-1963, dSim2/src/spinSystem.cpp:857-895),
with the steps replayed from a file (dsim3_set_replay / dsim2_set_replay).  The
result must equal the oracle run on the reference's own arrays and initial
state bit for bit: per-spin collision counts, positions, magnitudes, phases,
compartments and fibers.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle as O
from scenarios import CylCase, MeshCase, draws

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "oracle", "_ref")
F = np.float32


@pytest.fixture(scope="module")
def dropins(engine):
    if not (os.path.exists(os.path.join(SRC, "src3", "spinSystem.cpp")) and
            os.path.exists(os.path.join(SRC, "src2", "spinSystem.cpp"))):
        pytest.skip("the reference's scratch sources (oracle/build_ref.py) are not in this tree")
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build_ref
    from dsim_gb300 import build
    return build_ref.build_dropin(build.LIB)


def _run(exe, **kw):
    p = subprocess.run([exe] + ["%s=%s" % (k, v) for k, v in kw.items()], capture_output=True, text=True,
                       timeout=600)
    assert p.returncode == 0, (p.returncode, p.stderr[-2000:])
    return O.read_dump(kw["out"])


@pytest.mark.parametrize("membranes,perm", [("AM", 0.05), ("G", 0.2)])
def test_reference_dsim3_host_code_on_libdsim3(dropins, tmp_path, membranes, perm):
    from dsim_gb300.engine import grad_scaled, phase_constant
    case = MeshCase(tmp_path, membranes=membranes, permeability=perm, N=1200)
    iters, G, dt, gamma = 40, (40.0, -20.0, 60.0), 0.01, 42576.0
    d = draws(iters, case.N, seed=77)
    dpath = str(tmp_path / "draws.f32")
    np.ascontiguousarray(d).tofile(dpath)
    out = str(tmp_path / "dropin3.dump")
    r = _run(dropins[0], mesh=case.path, out=out, N=case.N, seed=5, spaceScale=case.spaceScale, dt=dt,
             extraAdc=2.0, myelinAdc=0.2, intraAdc=2.0, perm=perm, extraT2=80, myelinT2=7.5, intraT2=70,
             startBox=0.9, gx=G[0], gy=G[1], gz=G[2], gamma=gamma, iters=iters, reflType=1, draws=dpath)
    assert list(r["status"]) == [0, 0]
    n, n3, maxtpc = [int(x) for x in r["grid"]]
    p = O.params3(r["stdDevs"], r["T2"], perm, dt, n, maxtpc)
    mag, ph, comp, fib = O.spin_fields(r["spins0"])
    pos = r["pos0"].copy()
    cnt = np.zeros(2 * case.N, np.uint32)
    capped, _ = O.integrate3(p, pos, np.zeros(2 * case.N, np.uint32), mag, ph, comp, fib, r["vertices"],
                             r["helpers"], r["triInfo"], r["cubeCounter"], r["trianglesInCubes"],
                             grad_scaled(G, case.spaceScale), phase_constant(gamma, dt), iters, draws=d, counts=cnt)
    assert capped == 0
    gm, gph, gcomp, gfib = O.spin_fields(r["spins1"])
    assert cnt.reshape(-1, 2)[:, 0].sum() > 0 and cnt.reshape(-1, 2)[:, 1].sum() > 0
    assert np.array_equal(r["counts"], cnt)
    assert np.array_equal(r["pos1"].view(np.uint32), pos.view(np.uint32))
    assert np.array_equal(gm.view(np.uint32), mag.view(np.uint32))
    assert np.array_equal(gph.view(np.uint32), ph.view(np.uint32))
    assert np.array_equal(gcomp, comp) and np.array_equal(gfib, fib)
    assert len(np.unique(comp)) > 1


def test_reference_dsim2_host_code_on_libdsim2(dropins, tmp_path):
    """Single-membrane fibers (inner radius proportion 1): the reference's
    seed record (assignSeeds, dSim2/src/spinSystem.cpp:1129-1151) tells a GPU
    step only whether a spin is inside a fiber, which is its whole region when
    there is no myelin shell."""
    import ctypes as C
    case = CylCase(tmp_path, N=2000, permeability=0.05, inner=1.0)
    iters, G, dt, gamma, ss = 50, (80.0, 30.0, 0.0), 0.01, 42576.0, F(case.spaceScale)
    d = draws(iters, case.N, seed=78)
    dpath = str(tmp_path / "draws.f32")
    np.ascontiguousarray(d).tofile(dpath)
    out = str(tmp_path / "dropin2.dump")
    r = _run(dropins[1], fibers=case.path, out=out, N=case.N, seed=6, spaceScale=case.spaceScale, dt=dt,
             extraAdc=2.0, intraAdc=2.0, myelinAdc=0.2, extraT2=80, intraT2=70, myelinT2=8, perm=0.05, inner=1.0,
             gx=G[0], gy=G[1], gz=G[2], gamma=gamma, iters=iters, draws=dpath)
    assert list(r["status"]) == [0, 0]
    n, n3, maxfpc = [int(x) for x in r["grid"]]
    P = O.Params2()
    P.intraAdcScaled = F(2.0) / (ss * ss)
    P.extraAdcScaled = F(2.0) / (ss * ss)
    P.myelinAdcScaled = F(0.2) / (ss * ss)
    P.T2fiber, P.T2myelin, P.T2outside = 70.0, 8.0, 80.0
    P.permeability, P.innerRadiusProportion, P.spinRadius, P.deltaTime = 0.05, 1.0, 0.005, dt
    P.numCubes, P.maxFibersPerCube, P.cubeLength = n, maxfpc, float(r["cubeLength"][0])
    # update(): gradScaled = G * (1e-9f * spaceScale), phaseConstant = TWOPI * gamma * dt, in float
    gs = (np.array(G, F) * (F(1e-9) * ss)).astype(F)
    pc = F(6.28318530717959) * F(gamma) * F(dt)
    pos4, seed4, par = r["pos0"].copy(), r["seed0"].copy(), r["params0"].copy()
    cnt = np.zeros(2 * case.N, np.uint32)
    O.lib().or2_integrate(C.byref(P), case.N, pos4, seed4, par, r["fiberPos"], r["cubeCounter"], r["cubes"],
                          float(gs[0]), float(gs[1]), float(gs[2]), float(pc), iters,
                          np.ascontiguousarray(d.reshape(-1)), None, cnt)
    g4 = r["pos1"].reshape(-1, 4)
    gseed = r["seed1"].reshape(-1, 4)
    par = par.reshape(-1, 5)
    assert cnt.reshape(-1, 2)[:, 0].sum() > 0
    assert np.array_equal(r["counts"], cnt)
    assert np.array_equal(g4[:, :3].view(np.uint32), pos4.reshape(-1, 4)[:, :3].view(np.uint32))
    assert np.array_equal(g4[:, 3].view(np.uint32), par[:, 1].view(np.uint32))      # phase (pos.w on the GPU)
    assert np.array_equal(gseed[:, 2] - 1, par[:, 3].astype(np.uint32))              # region
    inside = par[:, 3] < 2
    assert np.array_equal(gseed[inside, 3], par[inside, 2].astype(np.uint32))       # fiber of inside spins
    assert inside.any() and (~inside).any()
