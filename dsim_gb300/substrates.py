"""Seeded synthetic substrates in the reference's input formats.

* beaded_tubes(): tessellated axons (rings of vertices, two triangles per quad)
  written as the dSim3 mesh fiber file (V / T / A<k> / M<k> / G<k> blocks,
  read by SpinSystem::initFibers, dSim3/src/spinSystem.cpp:290-673).  The
  ring/quad tessellation and end caps follow the construction of the
  reference's MATLAB generator (dSim3/fiberGeneration/dSimGetFiberTriangles.m:
  side triangles, then caps when the tube is closed), written here from its
  description.
* packed_cylinders(): parallel cylinders written as the dSim2 cylinder file
  (x y z r per line, INF on the axis; dSim2/src/spinSystem.cpp:323-385).

The reference's own benchmark substrates are not available (its .fmf meshes
are not in the repository), so these generators stand in for them with the
shapes, sizes and distributions of the benchmark configurations.
"""
import numpy as np


# --------------------------------------------------------------------------
# packing of disks in a square (positions in um)
# --------------------------------------------------------------------------
def _relax_disks(radii, half, rng, gap=0.02, iters=4000, margin=True):
    """Place disks of `radii` in [-half, half]^2 without overlap: random start,
    then iterative pairwise separation (soft-disk relaxation)."""
    n = len(radii)
    lo = -half + (radii if margin else np.zeros(n))
    hi = half - (radii if margin else np.zeros(n))
    pos = rng.uniform(0.0, 1.0, size=(n, 2)) * (hi - lo)[:, None] + lo[:, None]
    for _ in range(iters):
        d = pos[:, None, :] - pos[None, :, :]
        dist = np.sqrt((d ** 2).sum(-1)) + np.eye(n)
        need = radii[:, None] + radii[None, :] + gap
        ov = np.maximum(need - dist, 0.0)
        np.fill_diagonal(ov, 0.0)
        if ov.max() <= 1e-9:
            break
        push = (d / dist[..., None]) * (0.5 * ov)[..., None]
        pos += push.sum(1)
        if margin:
            pos = np.clip(pos, lo[:, None], hi[:, None])
    d = pos[:, None, :] - pos[None, :, :]
    dist = np.sqrt((d ** 2).sum(-1)) + np.eye(n) * 1e9
    overlap = bool((dist < radii[:, None] + radii[None, :]).any())
    return pos, overlap


def packed_cylinders(n=64, shape=5.0, mean=1.0, cell=20.0, fraction=0.5, seed=1):
    """n parallel z-cylinders, radii ~ Gamma(shape, mean/shape) rescaled so that
    the area fraction in the cell x cell square is `fraction`; packed inside the
    square (the reference drops cylinders that cross the box,
    dSim2/src/spinSystem.cpp:338-343).  Returns (xy[n,2], r[n]) in um."""
    rng = np.random.default_rng(seed)
    r = rng.gamma(shape, mean / shape, size=n)
    r *= np.sqrt(fraction * cell * cell / (np.pi * (r ** 2).sum()))
    order = np.argsort(-r)
    r = r[order]
    xy, overlap = _relax_disks(r, cell / 2.0, rng)
    if overlap:
        raise RuntimeError("cylinder packing did not converge")
    return xy, r


def write_cylinder_file(path, xy, r, axis="z"):
    """dSim2 cylinder file: one 'x y z r' line per fiber, INF on the axis."""
    with open(path, "w") as f:
        for (x, y), rr in zip(xy, r):
            if axis == "z":
                f.write("%.6f %.6f INF %.6f\n" % (x, y, rr))
            elif axis == "x":
                f.write("INF %.6f %.6f %.6f\n" % (x, y, rr))
            else:
                f.write("%.6f INF %.6f %.6f\n" % (x, y, rr))


def cylinders_normalised(xy, r, spaceScale):
    """fiberPos {x, y, 2.0, r^2} in normalised units, as initFibers(FILE*) stores."""
    F = np.float32
    ss = F(spaceScale)
    out = np.zeros((len(r), 4), F)
    out[:, 0] = xy[:, 0].astype(F) / ss
    out[:, 1] = xy[:, 1].astype(F) / ss
    out[:, 2] = F(2.0)
    rn = r.astype(F) / ss
    out[:, 3] = rn * rn
    return out.reshape(-1), float(rn.max())


# --------------------------------------------------------------------------
# tessellated tubes
# --------------------------------------------------------------------------
def tube_mesh(cx, cy, radius_fn, z0, z1, ring_spacing, verts_per_ring, closed=False, v_offset=0):
    """Vertices and triangles of one tube along z.  radius_fn(z) gives the
    radius of each ring; quads between rings are split into two triangles.
    With closed=True a centre vertex closes each end with a triangle fan."""
    nring = int(round((z1 - z0) / ring_spacing)) + 1
    z = np.linspace(z0, z1, nring)
    ang = 2 * np.pi * np.arange(verts_per_ring) / verts_per_ring
    rr = radius_fn(z)
    vx = cx + rr[:, None] * np.cos(ang)[None, :]
    vy = cy + rr[:, None] * np.sin(ang)[None, :]
    vz = np.repeat(z[:, None], verts_per_ring, 1)
    V = np.stack([vx, vy, vz], -1).reshape(-1, 3)
    k = np.arange(verts_per_ring)
    kn = (k + 1) % verts_per_ring
    tris = []
    for i in range(nring - 1):
        a = i * verts_per_ring + k
        b = i * verts_per_ring + kn
        c = (i + 1) * verts_per_ring + k
        d = (i + 1) * verts_per_ring + kn
        tris.append(np.stack([a, b, d], -1))
        tris.append(np.stack([a, d, c], -1))
    T = np.concatenate(tris, 0)
    if closed:
        c0 = len(V)
        V = np.concatenate([V, [[cx, cy, z0], [cx, cy, z1]]], 0)
        last = (nring - 1) * verts_per_ring
        cap0 = np.stack([np.full(verts_per_ring, c0), kn, k], -1)
        cap1 = np.stack([np.full(verts_per_ring, c0 + 1), last + k, last + kn], -1)
        T = np.concatenate([T, cap0, cap1], 0)
    return V, T + v_offset


def beaded_tubes(n_axons=400, verts_per_ring=32, ring_spacing=0.5, length=50.0, box=50.0,
                 radius_median=1.0, radius_sigma=0.4, radius_clip=(0.5, 3.0), bead_amp=0.2,
                 bead_period=10.0, seed=1, closed=False, membranes="G", z_range=None,
                 allow_overlap=True):
    """Beaded axons r(z) = r0 (1 + a sin(2 pi z / P)) with r0 ~ LogNormal(median,
    sigma) clipped, placed in the box x box square (um), z in [-length/2,
    length/2].  membranes "G": one glia-type membrane per axon (compartments
    0 <-> 3); "AM": axon (A) and myelin (M) membranes at r and 1.25 r.
    Returns dict(vertices[V,3] um, trgls[T,3], membrane[T], fiber[T], centres,
    radii, overlap)."""
    rng = np.random.default_rng(seed)
    r0 = np.clip(rng.lognormal(np.log(radius_median), radius_sigma, n_axons), *radius_clip)
    rmax = r0 * (1 + abs(bead_amp)) * (1.25 if membranes == "AM" else 1.0)
    xy, overlap = _relax_disks(rmax, box / 2.0, rng, gap=0.05, iters=300 if allow_overlap else 3000)
    if overlap and not allow_overlap:
        raise RuntimeError("tube packing did not converge")
    z0, z1 = (-length / 2.0, length / 2.0) if z_range is None else z_range
    Vs, Ts, mem, fib = [], [], [], []
    nv = 0
    for i in range(n_axons):
        layers = [(2, 1.0)] if membranes == "G" else [(0, 1.0), (1, 1.25)]
        for (mtype, scale) in layers:
            rf = (lambda z, r=r0[i], s=scale: s * r * (1 + bead_amp * np.sin(2 * np.pi * z / bead_period)))
            V, T = tube_mesh(xy[i, 0], xy[i, 1], rf, z0, z1, ring_spacing, verts_per_ring,
                             closed=closed, v_offset=nv)
            Vs.append(V); Ts.append(T)
            mem.append(np.full(len(T), mtype, np.uint32))
            fib.append(np.full(len(T), i, np.uint32))
            nv += len(V)
    return dict(vertices=np.concatenate(Vs).astype(np.float32),
                trgls=np.concatenate(Ts).astype(np.uint32),
                membrane=np.concatenate(mem), fiber=np.concatenate(fib),
                centres=xy, radii=r0, overlap=overlap)


def write_mesh_file(path, mesh):
    """dSim3 mesh fiber file: V block, T block, then per fiber and membrane a
    block 'A<k>' / 'M<k>' / 'G<k>' listing its triangle indices (ascending).
    Vertices are written with 9 significant digits, so a float32 vertex reads
    back as the same float."""
    V, T = np.asarray(mesh["vertices"]), np.asarray(mesh["trgls"])
    mem, fib = np.asarray(mesh["membrane"]), np.asarray(mesh["fiber"])
    letters = {0: "A", 1: "M", 2: "G"}
    order = np.lexsort((np.arange(len(fib)), mem, fib))
    key = fib[order].astype(np.int64) * 4 + mem[order]
    cuts = np.nonzero(np.diff(key))[0] + 1
    with open(path, "w") as f:
        f.write("V\n")
        np.savetxt(f, V, fmt="%.9g")
        f.write("T\n")
        np.savetxt(f, T, fmt="%d")
        for idx in np.split(order, cuts):
            if len(idx) == 0:
                continue
            f.write("%s%d\n" % (letters[int(mem[idx[0]])], int(fib[idx[0]])))
            f.write("\n".join(map(str, idx.tolist())) + "\n")
