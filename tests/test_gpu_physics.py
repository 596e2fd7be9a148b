"""GPU checks of the generator, the ensemble signal and free diffusion.

* Philox4x32-10 words on the GPU equal the oracle's (which matches the
  published known-answer vectors, tests/test_cpu_oracle.py).
* The Box-Muller mapping of those words equals a float64 evaluation within
  2e-6 (CUDA's logf / sincospif are not the host's functions).
* The device FP64 signal reduction equals the oracle's getMrSignal.
* Free diffusion: the PGSE signal equals exp(-b D),
  b = (2 pi gamma G delta)^2 (Delta - delta/3) (dSim3/src/diffusion.cpp:317),
  in the exact form of the discrete walk (below), within 3 Monte-Carlo
  standard errors and no other slack.
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def test_philox_words_match_oracle_and_box_muller(engine):
    from dsim_gb300._lib import native, check
    n = 4096
    seed = 0x1234_5678_9ABC_DEF0
    raw = np.zeros(4 * n, np.uint32)
    dr = np.zeros(4 * n, np.float32)
    check(native().dsim_rng_draws(seed, 100, 77, 5, n, raw, dr))
    raw = raw.reshape(-1, 4)
    for i in (0, 1, 17, 4095):
        ref = O.philox([100 + i, 77, 0, 5], [seed & 0xFFFFFFFF, seed >> 32])
        assert np.array_equal(raw[i], ref)
    w = raw.astype(np.float64)
    u1 = w[:, 0] * 2.0 ** -32 + 2.0 ** -33
    u2 = np.floor(w[:, 1] / 256) * 2.0 ** -24
    u3 = w[:, 2] * 2.0 ** -32 + 2.0 ** -33
    u4 = (np.floor(w[:, 3] / 256) + 1) * 2.0 ** -24
    r1 = np.sqrt(-2 * np.log(u1))
    r2 = np.sqrt(-2 * np.log(u3))
    ref = np.stack([r1 * np.cos(2 * np.pi * u2), r1 * np.sin(2 * np.pi * u2),
                    r2 * np.cos(2 * np.pi * u4), u4], -1)
    got = dr.reshape(-1, 4).astype(np.float64)
    assert np.max(np.abs(got - ref)) < 2e-5
    assert np.array_equal(got[:, 3], u4)
    # moments of the normals
    z = got[:, :3].reshape(-1)
    assert abs(z.mean()) < 0.05 and abs(z.std() - 1) < 0.05


def test_signal_reduction_matches_oracle(engine):
    from dsim_gb300.engine import Spins, signal_from_sums
    rng = np.random.default_rng(4)
    N = 100_003
    pos = rng.uniform(-1, 1, 3 * N).astype(np.float32)
    mag = rng.uniform(0.5, 1.0, N).astype(np.float32)
    ph = rng.normal(0, 3, N).astype(np.float32)
    comp = rng.integers(0, 4, N).astype(np.uint8)
    s = Spins(N)
    s.set(pos, mag, ph, comp, np.zeros(N, np.uint16))
    got = signal_from_sums(s.signal())
    ref = O.signal3(mag, ph, comp)
    # the reference forms cos/sin products in float, the device in double
    assert np.allclose(got, ref, rtol=2e-6, atol=1e-7)
    sums = s.signal()
    assert sums[0, 2] == N and sums[1:, 2].sum() == N


def discrete_free_signal(grad_per_step, sigma, pc):
    """Expected signal of the discrete free walk x_t = x_0 + sigma sum_{s<=t} n_s
    with phase pc sum_t g_t . x_t.  For a balanced waveform (sum_t g_t = 0) the
    phase is pc sigma sum_s n_s . W_s, W_s = sum_{t>=s} g_t, a Gaussian of
    variance V = (pc sigma)^2 sum_s |W_s|^2, so E cos(phi) = exp(-V/2).  This
    is exp(-b D) with b in the form of the walk's own time steps."""
    g = np.asarray(grad_per_step, np.float64).reshape(-1, 3)
    assert np.allclose(g.sum(0), 0.0, atol=1e-12)
    W = np.cumsum(g[::-1], axis=0)[::-1]
    V = (float(pc) * float(sigma)) ** 2 * float((W ** 2).sum())
    return np.exp(-V / 2)


def free_se(S, N):
    """Standard error of mean cos(phi) for phi ~ N(0, V), E cos = S:
    Var cos = (1 + S^4)/2 - S^2 = (1 - S^2)^2 / 2."""
    return (1.0 - S * S) / np.sqrt(2.0 * N)


@pytest.mark.parametrize("G,direction", [(0.0, (1, 0, 0)), (40.0, (1, 0, 0)),
                                         (80.0, (0, 0, 1)), (80.0, (1, 1, 0))])
def test_free_diffusion_pgse_matches_exp_minus_bD(engine, G, direction):
    from dsim_gb300.engine import (Mesh, Spins, grad_scaled, mesh_params, mesh_run,
                                   phase_constant, signal_from_sums, std_devs)
    D, dt, delta, Delta = 2.0, 0.01, 10.0, 30.0
    spaceScale = 1000.0
    N = 1 << 20
    # a substrate with no triangles: free diffusion
    m = Mesh.from_arrays(np.zeros((3, 3), np.float32), np.zeros((0, 3), np.uint32), None, None,
                         spaceScale)
    rng = np.random.default_rng(2)
    s = Spins(N)
    s.set(rng.uniform(-0.3, 0.3, 3 * N).astype(np.float32), np.ones(N, np.float32),
          np.zeros(N, np.float32), np.zeros(N, np.uint8), np.full(N, 0xFFFF, np.uint16))
    sd = std_devs(D, D, D, spaceScale, dt)
    pc = phase_constant(42576.0, dt)
    p = mesh_params(sd, [1e30] * 4, 0.0, dt, pc)
    u = np.asarray(direction, np.float64)
    u = u / np.linalg.norm(u)
    g = grad_scaled(G * u, spaceScale)
    nd, nD = int(round(delta / dt)), int(round(Delta / dt))
    step = 0
    segs = ((g, nd), (np.zeros(3, np.float32), nD - nd), (-g, nd))
    for gg, n in segs:
        mesh_run(m, s, p, g=gg, iterations=n, seed=99, step0=step)
        step += n
    S = signal_from_sums(s.signal())[0]
    assert s.status() == 0
    gps = np.concatenate([np.repeat(np.asarray(gg, np.float64)[None, :], n, 0) for gg, n in segs])
    expect = discrete_free_signal(gps, sd[0], pc)
    b = (2 * np.pi * 42576.0 * G * 1e-9 * delta) ** 2 * (Delta - delta / 3.0)
    assert abs(expect - np.exp(-b * D)) < 5e-3              # the continuous closed form
    assert abs(S - expect) <= 3 * free_se(expect, N), (S, expect, b)
