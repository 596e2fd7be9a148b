"""The cylinder fine filter grid's lists (dsim_cyl_fine_lists: the host code
whose output dsim_cyl_set_fine uploads), checked by brute force on the CPU.

A spin outside every fiber tests, at a point p, the entries of p's grid-cell
list; only an entry whose fiber holds p (float d^2 <= r^2, computed as the
step computes it) can change anything.  For points anywhere a step can test
-- uniform in and past the box, on fine-cell and grid-cell boundaries, on
fiber surfaces and a float step either side of them -- every such entry must
be in the fine list of p's fine cell, and each fine list must be an
increasing run of list positions.  The point-to-cell arithmetic below is the
step kernel's, in float32 (numpy rounds every operation to float32, as the
kernel does without contraction)."""
import ctypes as C
import math

import numpy as np
import pytest

import oracle as O
from dsim_gb300 import substrates as S

F = np.float32


def _mixed_fibers(seed, per_axis=24):
    rng = np.random.default_rng(seed)
    rows = []
    for axis in (0, 1, 2):
        for _ in range(per_axis):
            c = rng.uniform(-0.9, 0.9, 3)
            r = rng.uniform(0.03, 0.12)
            c[axis] = 2.0
            rows.append([c[0], c[1], c[2], r * r])
    fp = np.array(rows, F).reshape(-1)
    return fp, float(np.sqrt(fp.reshape(-1, 4)[:, 3].max()))


def _packed(n):
    cell = 20.0 * math.sqrt(n / 64.0)
    xy, r = S.packed_cylinders(n=n, cell=cell, fraction=0.5, seed=1)
    fp, rmax = S.cylinders_normalised(xy, r, cell / 2.0)
    return np.ascontiguousarray(fp, F).reshape(-1), float(rmax)


def _fine_lists(lib, fp, grid, k):
    cc, cubes, n, maxfpc, L = grid
    nfine = (n * k) ** 3
    start = np.zeros(nfine + 1, np.uint32)
    ent = C.c_uint64(0)
    rc = lib.dsim_cyl_fine_lists(fp, len(fp) // 4, n, maxfpc, float(L), cc, cubes, k, start, None, 0, C.byref(ent))
    assert rc == 0
    pos = np.zeros(max(1, ent.value), np.uint32)
    rc = lib.dsim_cyl_fine_lists(fp, len(fp) // 4, n, maxfpc, float(L), cc, cubes, k, start, pos, len(pos),
                                 C.byref(ent))
    assert rc == 0
    return start, pos[:ent.value]


def _cells(p, n, k, L):
    """Grid cell (the reference's calcCubeHash rule) and fine cell of float32 points."""
    L = F(L)
    inv = F(1.0) / L
    hi = F(n - 1)
    c = np.clip(np.floor((p + F(1.0)) * inv), F(0.0), hi)
    cube = ((F(n * n) * c[:, 2]).astype(np.int64) + (F(n) * c[:, 1]).astype(np.int64) + c[:, 0].astype(np.int64))
    cx, cy, cz = cube % n, (cube // n) % n, cube // (n * n)
    finv = F(k) / L
    s = np.floor((p + F(1.0)) * finv) - np.stack([cx * k, cy * k, cz * k], 1).astype(F)
    s = np.clip(s, F(0.0), F(k - 1)).astype(np.int64)
    nk = n * k
    fc = ((cz * k + s[:, 2]) * nk + (cy * k + s[:, 1])) * nk + cx * k + s[:, 0]
    return cube, fc


def _dist_sq(p, f):
    """The step's distance of points p (m x 3) to fibers f (m x e x 4), float32."""
    px, py, pz = (p[:, a][:, None] for a in range(3))
    fx, fy, fz = f[..., 0], f[..., 1], f[..., 2]
    dxy = (px - fx) * (px - fx) + (py - fy) * (py - fy)
    dyz = (pz - fz) * (pz - fz) + (py - fy) * (py - fy)
    dxz = (px - fx) * (px - fx) + (pz - fz) * (pz - fz)
    return np.where(fx == F(2.0), dyz, np.where(fz == F(2.0), dxy, dxz))


def _points(fp, n, k, L, rng, m=60000):
    f4 = fp.reshape(-1, 4)
    pts = [rng.uniform(-1.05, 1.05, (m, 3)).astype(F)]
    # on fine-cell (and so grid-cell) boundaries, one or more coordinates
    Lf = F(L) / F(k)
    b = rng.uniform(-0.99, 0.99, (m, 3)).astype(F)
    g = rng.integers(0, n * k + 1, (m, 3))
    onb = (F(-1.0) + g.astype(F) * Lf).astype(F)
    mask = rng.random((m, 3)) < 0.5
    mask[np.arange(m), rng.integers(0, 3, m)] = True
    pts.append(np.where(mask, onb, b).astype(F))
    # on fiber surfaces, and one float step either side
    sel = rng.integers(0, len(f4), m)
    ang = rng.uniform(0, 2 * np.pi, m)
    r = np.sqrt(f4[sel, 3].astype(np.float64))
    surf = rng.uniform(-0.99, 0.99, (m, 3))
    for i in range(m):
        f = f4[sel[i]]
        axes = (1, 2) if f[0] == 2.0 else ((0, 1) if f[2] == 2.0 else (0, 2))
        surf[i, axes[0]] = f[axes[0]] + r[i] * np.cos(ang[i])
        surf[i, axes[1]] = f[axes[1]] + r[i] * np.sin(ang[i])
    surf = surf.astype(F)
    pts += [surf, np.nextafter(surf, F(2.0)), np.nextafter(surf, F(-2.0))]
    # past the box (a proposed position before the clamp)
    far = rng.uniform(-1.0, 1.0, (m // 4, 3)).astype(F)
    far[:, rng.integers(0, 3)] = rng.choice([F(-1.3), F(1.3)], m // 4)
    pts.append(far)
    return np.concatenate(pts)


@pytest.mark.parametrize("which,k", [("packed64", 10), ("packed64", 3), ("packed256", 15), ("mixed", 2),
                                     ("mixed", 7), ("mixed", 16)])
def test_fine_lists_hold_every_entry_that_can_act(engine, which, k):
    lib = engine.native()
    fp, maxR = {"packed64": lambda: _packed(64), "packed256": lambda: _packed(256),
                "mixed": lambda: _mixed_fibers(5)}[which]()
    grid = O.build_grid2(fp, maxR)
    cc, cubes, n, maxfpc, L = grid
    start, pos = _fine_lists(lib, fp, grid, k)
    nfine = (n * k) ** 3
    assert start[0] == 0 and np.all(np.diff(start.astype(np.int64)) >= 0) and start[-1] == len(pos)
    # each fine list: strictly increasing positions inside its grid cell's list
    nk = n * k
    fcs = np.arange(nfine)
    gx, gy, gz = fcs % nk, (fcs // nk) % nk, fcs // (nk * nk)
    parent = ((gz // k) * n + gy // k) * n + gx // k
    lens = np.diff(start.astype(np.int64))
    owner = np.repeat(fcs, lens)
    assert np.all(pos < cc[parent[owner]])
    same = owner[1:] == owner[:-1]
    assert np.all(pos[1:][same] > pos[:-1][same])
    # membership table: in_fine[fine cell, list position]
    in_fine = np.zeros((nfine, maxfpc), bool)
    in_fine[owner, pos] = True
    assert len(pos) < cc[parent].sum()      # it filters
    rng = np.random.default_rng(k + len(fp))
    p = _points(fp, n, k, L, rng)
    cube, fc = _cells(p, n, k, L)
    f4 = fp.reshape(-1, 4)
    acted = 0
    for lo in range(0, len(p), 20000):
        sl = slice(lo, lo + 20000)
        ent = cubes.reshape(-1, maxfpc)[cube[sl]]                 # m x maxfpc fiber indices
        valid = np.arange(maxfpc)[None, :] < cc[cube[sl]][:, None]
        f = f4[np.where(valid, ent, 0)]
        cur = _dist_sq(p[sl], f)
        act = valid & (cur <= f[..., 3])
        missing = act & ~in_fine[fc[sl]]
        assert not missing.any(), (which, k, np.argwhere(missing)[:5])
        acted += int(act.sum())
    # the check saw entries that act (fiber-surface points among them)
    assert acted > len(p) // 20


def test_fine_lists_reject_bad_grids(engine):
    lib = engine.native()
    fp, maxR = _mixed_fibers(5)
    cc, cubes, n, maxfpc, L = O.build_grid2(fp, maxR)
    ent = C.c_uint64(0)
    start = np.zeros((n * 4) ** 3 + 1, np.uint32)
    bad = cubes.copy()
    bad[0] = len(fp) // 4                     # names a fiber that does not exist
    cc1 = cc.copy()
    cc1[0] = max(cc1[0], 1)
    assert lib.dsim_cyl_fine_lists(fp, len(fp) // 4, n, maxfpc, float(L), cc1, bad, 4, start, None, 0,
                                   C.byref(ent)) != 0
    over = cc.copy()
    over[0] = maxfpc + 1                      # more entries than a cell holds
    assert lib.dsim_cyl_fine_lists(fp, len(fp) // 4, n, maxfpc, float(L), over, cubes, 4, start, None, 0,
                                   C.byref(ent)) != 0
    assert lib.dsim_cyl_fine_lists(fp, len(fp) // 4, n, maxfpc, float(L), cc, cubes, 1, start, None, 0,
                                   C.byref(ent)) != 0   # k < 2
    _, pos = _fine_lists(lib, fp, (cc, cubes, n, maxfpc, L), 4)
    short = np.zeros(max(1, len(pos) - 1), np.uint32)
    assert lib.dsim_cyl_fine_lists(fp, len(fp) // 4, n, maxfpc, float(L), cc, cubes, 4, start, short, len(short),
                                   C.byref(ent)) != 0   # capacity short


def test_fine_lists_keep_repeated_entries(engine):
    """A fiber listed twice in one cell (the reference's halo lines can do
    that) is tested twice by the reference; the fine lists keep both list
    positions, in order, wherever the fiber can act."""
    lib = engine.native()
    fp, maxR = _mixed_fibers(5)
    cc, cubes, n, maxfpc, L = O.build_grid2(fp, maxR)
    k = 4
    nk = n * k
    cell = int(np.argmax(cc))
    cx, cy, cz = cell % n, (cell // n) % n, cell // (n * n)
    # an entry of that cell whose fiber reaches into it (the reference's halo
    # also lists fibers that do not)
    start0, pos0 = _fine_lists(lib, fp, (cc, cubes, n, maxfpc, L), k)
    own = set()
    for sz in range(k):
        for sy in range(k):
            for sx in range(k):
                fc = ((cz * k + sz) * nk + (cy * k + sy)) * nk + cx * k + sx
                own.update(int(j) for j in pos0[start0[fc]:start0[fc + 1]])
    j0 = min(own)
    cc = cc.copy()
    cubes = cubes.copy().reshape(-1, maxfpc)
    assert cc[cell] < maxfpc
    cubes[cell, cc[cell]] = cubes[cell, j0]   # the same fiber again, at the end of the list
    cc[cell] += 1
    cubes = cubes.reshape(-1)
    start, pos = _fine_lists(lib, fp, (cc, cubes, n, maxfpc, L), k)
    seen_both = 0
    for sz in range(k):
        for sy in range(k):
            for sx in range(k):
                fc = ((cz * k + sz) * nk + (cy * k + sy)) * nk + cx * k + sx
                lst = pos[start[fc]:start[fc + 1]]
                has0, hasl = j0 in lst, (cc[cell] - 1) in lst
                assert has0 == hasl                  # the same fiber: both or neither
                seen_both += has0
                assert np.all(np.diff(lst.astype(np.int64)) > 0)
    assert seen_both > 0
