"""Seeded scenarios shared by the parity tests: small substrates written in
the reference's formats, initial spin states and replay draw streams."""
import os

import numpy as np

from dsim_gb300 import substrates as S
from dsim_gb300.engine import grad_scaled, phase_constant, std_devs

F = np.float32


def draws(iterations, N, seed):
    """Replay stream [iterations][N][4]: three standard normals and u in (0, 1]."""
    rng = np.random.default_rng(seed)
    d = np.empty((iterations, N, 4), F)
    d[..., :3] = rng.standard_normal((iterations, N, 3)).astype(F)
    d[..., 3] = (1.0 - rng.random((iterations, N))).astype(F)
    return d


class MeshCase:
    """Closed tessellated tubes with axon/myelin (AM) or glia (G) membranes."""

    def __init__(self, tmpdir, membranes="AM", N=1500, seed=5, spaceScale=10.0, n_axons=3,
                 verts=12, ring=1.0, permeability=0.05, D=2.0, dt=0.01, T2=(80.0, 70.0, 7.5, 60.0)):
        self.tube = S.beaded_tubes(n_axons=n_axons, verts_per_ring=verts, ring_spacing=ring,
                                   length=16.0, box=12.0, closed=True, membranes=membranes,
                                   seed=seed, allow_overlap=False, bead_period=8.0)
        self.path = os.path.join(str(tmpdir), "mesh_%s_%d.txt" % (membranes, seed))
        S.write_mesh_file(self.path, self.tube)
        self.spaceScale = spaceScale
        self.N = N
        rng = np.random.default_rng(seed + 100)
        pos = rng.uniform(-0.9, 0.9, (N, 3)).astype(F)
        self.pos = pos.reshape(-1).copy()
        self.comp, self.fiber = self._compartments(pos, membranes)
        self.mag = np.ones(N, F)
        self.phase = np.zeros(N, F)
        self.dt = F(dt)
        self.stdDevs = std_devs(D, D, 0.1 * D, spaceScale, dt)
        self.T2 = np.array(T2, F)
        self.permeability = F(permeability)
        self.g = grad_scaled([40.0, -20.0, 60.0], spaceScale)
        self.pc = phase_constant(42576.0, dt)

    def _compartments(self, pos, membranes):
        um = pos.astype(np.float64) * self.spaceScale
        comp = np.zeros(len(pos), np.uint8)
        fib = np.full(len(pos), 0xFFFF, np.uint16)
        for i, ((cx, cy), r0) in enumerate(zip(self.tube["centres"], self.tube["radii"])):
            z = um[:, 2]
            r = r0 * (1 + 0.2 * np.sin(2 * np.pi * z / 8.0))
            d = np.hypot(um[:, 0] - cx, um[:, 1] - cy)
            inside_z = np.abs(z) < 8.0
            if membranes == "G":
                sel = inside_z & (d < 0.9 * r)
                comp[sel] = 3
                fib[sel] = i
            else:
                ax = inside_z & (d < 0.9 * r)
                my = inside_z & (d > 1.1 * r) & (d < 0.9 * 1.25 * r)
                comp[ax] = 1
                comp[my] = 2
                fib[ax | my] = i
        return comp, fib


class CylCase:
    """Packed parallel cylinders (dSim2 cylinder file)."""

    def __init__(self, tmpdir, N=2000, seed=1, spaceScale=10.0, n=64, fraction=0.5,
                 permeability=0.02, inner=0.7, D=2.0, dt=0.01):
        self.xy, self.r = S.packed_cylinders(n=n, cell=19.0, fraction=fraction, seed=seed)
        self.path = os.path.join(str(tmpdir), "cyl_%d.fibers" % seed)
        S.write_cylinder_file(self.path, self.xy, self.r)
        self.spaceScale = spaceScale
        self.N = N
        rng = np.random.default_rng(seed + 7)
        self.pos = rng.uniform(-0.95, 0.95, (N, 3)).astype(F).reshape(-1)
        self.permeability = F(permeability)
        self.inner = F(inner)
        self.D = D
        self.dt = F(dt)
        self.g = grad_scaled([80.0, 0.0, 0.0], spaceScale)
        self.pc = phase_constant(42576.0, dt)
