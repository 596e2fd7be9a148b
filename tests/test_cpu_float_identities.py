"""The float identities the step kernels use in place of conversion
instructions, checked here in IEEE float32 arithmetic (numpy rounds each
operation to nearest, as the kernels' __fadd_rn / __fsub_rn do):

* floor_small (common.cuh): r = (t + 1.5*2^23) - 1.5*2^23, then r - 1 where
  r > t, equals floorf(t) for |t| < 2^22 (a zero result is +0);
* uint_small: the bits of f + 2^23 minus 0x4B000000 equal (uint32_t)f for an
  integer-valued f in [0, 2^23).
The grid and lattice coordinates of the mesh and cylinder steps depend on
these being exact."""
import numpy as np

F = np.float32
M = F(12582912.0)      # 1.5 * 2^23


def floor_small(t):
    t = np.asarray(t, F)
    r = (t + M) - M
    return np.where(r > t, r - F(1), r).astype(F)


def uint_small(f):
    f = np.asarray(f, F)
    return ((f + F(8388608.0)).view(np.uint32) - np.uint32(0x4B000000)).astype(np.uint32)


def test_floor_small_equals_floorf():
    rng = np.random.default_rng(3)
    t = np.concatenate([
        rng.uniform(-4.0, 4.0, 400_000), rng.uniform(-300.0, 300.0, 400_000),
        rng.uniform(-(2.0 ** 22) + 1, 2.0 ** 22 - 1, 200_000),
        np.arange(-64, 64) * 0.5, np.arange(-64, 64) * 0.25,              # ties and quarters
        np.nextafter(np.arange(-20, 20, dtype=F), F(np.inf)),
        np.nextafter(np.arange(-20, 20, dtype=F), F(-np.inf)),
        [0.0, -0.0, 1e-30, -1e-30, 0.9999999, -0.9999999],
    ]).astype(F)
    want = np.floor(t)
    got = floor_small(t)
    assert np.array_equal(got, want)          # values (a -0 floor comes back as +0)
    # as used: grid coordinates (p + 1) * inv for p in the box, and lattice steps p * 16
    p = rng.uniform(-1.2, 1.2, 200_000).astype(F)
    for inv in (F(1.0 / (2.0 / 112)), F(25.0), F(56.0), F(1.0 / F(0.04))):
        u = ((p + F(1)) * inv).astype(F)
        assert np.array_equal(floor_small(u), np.floor(u))
    assert np.array_equal(floor_small(p * F(16)), np.floor(p * F(16)))


def test_uint_small_equals_conversion():
    f = np.concatenate([np.arange(0, 5000), np.arange(2 ** 23 - 5000, 2 ** 23)]).astype(F)
    assert np.array_equal(uint_small(f), f.astype(np.uint32))
