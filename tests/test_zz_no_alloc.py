"""dsim_signal_noalloc: the ensemble signal over the reference's own device
spin arrays, with scratch from a fixed array inside libdsim_gb300.so instead
of an allocation.  Called through the C-ABI and compared with dsim_signal on
the same spins (FP64 sums; the two add in different orders, so the tolerance
is relative 1e-12 on X and Y, exact on counts).  Collected last so it also
runs after every other GPU test in the same process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12
DSIM_SIGNAL_DSIM3, DSIM_SIGNAL_DSIM2 = 1, 2
DSIM_ETOOLARGE = -6
MAX_SPINS = 16_777_216


def _close(a, b):
    a = np.asarray(a).reshape(5, 3); b = np.asarray(b).reshape(5, 3)
    assert np.array_equal(a[:, 2], b[:, 2]), (a[:, 2], b[:, 2])
    scale = np.maximum(b[:, 2], 1.0)
    assert np.all(np.abs(a[:, :2] - b[:, :2]) <= RTOL * scale[:, None]), (a, b)


class _Dev:
    """Device buffers through the dSim3 C-ABI (the caller owns them)."""

    def __init__(self):
        from dsim_gb300 import _lib
        self.L = _lib.abi3()
        self.bufs = []

    def put(self, arr):
        arr = np.ascontiguousarray(arr)
        p = C.c_void_p()
        self.L.allocateArray(C.byref(p), max(arr.nbytes, 16))
        assert p.value, "allocateArray failed"
        self.L.copyArrayToDevice(p, arr.ctypes.data, 0, arr.nbytes)
        self.bufs.append(p)
        return p

    def get(self, p, like):
        out = np.zeros_like(like)
        self.L.copyArrayFromDevice(out.ctypes.data, p, 0, out.nbytes)
        return out

    def free(self):
        for p in self.bufs:
            self.L.freeArray(p)


def _spins(N, seed):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-1, 1, (N, 3)).astype(np.float32)
    mag = rng.uniform(0.2, 1.0, N).astype(np.float32)
    ph = rng.uniform(-40, 40, N).astype(np.float32)
    comp = rng.integers(0, 4, N).astype(np.uint8)
    fib = rng.integers(0, 300, N).astype(np.uint16)
    return pos, mag, ph, comp, fib


@pytest.mark.parametrize("N", [1, 2047, 2048, 300_001])
def test_noalloc_signal_dsim3_arrays_match_dsim_signal(engine, N):
    from dsim_gb300 import _lib
    from dsim_gb300.engine import Spins
    L = _lib.native()
    pos, mag, ph, comp, fib = _spins(N, seed=N)
    s = Spins(N)
    s.set(pos, mag, ph, comp, fib)
    rec = np.zeros(N, np.dtype([("mag", "<f4"), ("phase", "<f4"), ("comp", "u1"), ("pad", "u1"),
                                ("fiber", "<u2")]))
    rec["mag"], rec["phase"], rec["comp"], rec["fiber"] = mag, ph, comp, fib
    d = _Dev()
    try:
        dpos, drec = d.put(pos), d.put(rec)
        dout = d.put(np.zeros(15, np.float64))
        for region in (0.0, 0.8):
            want = s.signal(region)
            got = []
            for _ in range(2):  # two calls in a row reuse the same scratch
                rc = L.dsim_signal_noalloc(dpos, drec, N, DSIM_SIGNAL_DSIM3, region, dout, None)
                assert rc == 0, L.dsim_last_error()
                got.append(d.get(dout, np.zeros(15, np.float64)))
            _close(got[0], want)
            _close(got[1], want)
            assert np.array_equal(got[0], got[1])
    finally:
        d.free()


def test_noalloc_signal_dsim2_arrays_match_dsim_signal(engine):
    from dsim_gb300 import _lib
    from dsim_gb300.engine import Spins
    L = _lib.native()
    N = 100_003
    pos, _, ph, _, _ = _spins(N, seed=7)
    imo = np.random.default_rng(8).integers(0, 3, N).astype(np.uint32)
    s = Spins(N)
    s.set_cyl(pos, np.ones(N, np.float32), ph, imo, np.zeros(N, np.uint32))
    pos4 = np.concatenate([pos, ph[:, None]], axis=1).astype(np.float32)
    seeds = np.zeros((N, 4), np.uint32)
    seeds[:, 2] = imo + 1
    d = _Dev()
    try:
        dpos, dseed = d.put(pos4), d.put(seeds)
        dout = d.put(np.zeros(15, np.float64))
        for region in (0.0, 0.8):
            want = s.signal(region)
            for _ in range(2):
                rc = L.dsim_signal_noalloc(dpos, dseed, N, DSIM_SIGNAL_DSIM2, region, dout, None)
                assert rc == 0, L.dsim_last_error()
                _close(d.get(dout, np.zeros(15, np.float64)), want)
    finally:
        d.free()


def test_noalloc_signal_dsim2_fresh_reference_seeds(engine):
    """Seed records as the reference's assignSeeds leaves them before the
    first step (dSim2/src/spinSystem.cpp:1129-1151): word 2 = 0, word 3 = the
    nearest fiber for a spin inside one, UINT_MAX outside.  They must read as
    core (0) and outside (2), as the step kernel reads them."""
    from dsim_gb300 import _lib
    from dsim_gb300.engine import Spins
    L = _lib.native()
    N = 70_001
    pos, _, ph, _, _ = _spins(N, seed=11)
    rng = np.random.default_rng(12)
    inside = rng.random(N) < 0.4
    w3 = np.where(inside, rng.integers(0, 64, N), 0xFFFFFFFF).astype(np.uint32)
    s = Spins(N)
    s.set_cyl(pos, np.ones(N, np.float32), ph, np.where(inside, 0, 2).astype(np.uint32),
              np.where(inside, w3, 0).astype(np.uint32))
    pos4 = np.concatenate([pos, ph[:, None]], axis=1).astype(np.float32)
    seeds = np.zeros((N, 4), np.uint32)
    seeds[:, :2] = rng.integers(1, 2 ** 32 - 1, (N, 2), dtype=np.uint64).astype(np.uint32)
    seeds[:, 3] = w3
    d = _Dev()
    try:
        dpos, dseed = d.put(pos4), d.put(seeds)
        dout = d.put(np.zeros(15, np.float64))
        for region in (0.0, 0.8):
            want = s.signal(region)
            assert want[2, 2] == 0 and want[1, 2] > 0 and want[3, 2] > 0
            for _ in range(2):
                rc = L.dsim_signal_noalloc(dpos, dseed, N, DSIM_SIGNAL_DSIM2, region, dout, None)
                assert rc == 0, L.dsim_last_error()
                _close(d.get(dout, np.zeros(15, np.float64)), want)
    finally:
        d.free()


def test_noalloc_signal_counts_compartments_above_3_in_the_total_only(engine):
    """The reference sizes its sums by its four compartments
    (dSim3/src/spinSystem.cpp:1452-1500); an index above 3 is counted in the
    total and in no compartment, so the caller can see it as the difference."""
    from dsim_gb300 import _lib
    L = _lib.native()
    N = 50_000
    pos, mag, ph, _, fib = _spins(N, seed=13)
    comp = np.random.default_rng(14).integers(0, 7, N).astype(np.uint8)
    rec = np.zeros(N, np.dtype([("mag", "<f4"), ("phase", "<f4"), ("comp", "u1"), ("pad", "u1"),
                                ("fiber", "<u2")]))
    rec["mag"], rec["phase"], rec["comp"], rec["fiber"] = mag, ph, comp, fib
    X = mag.astype(np.float64) * np.cos(ph.astype(np.float64))
    Y = mag.astype(np.float64) * np.sin(ph.astype(np.float64))
    want = np.zeros((5, 3))
    want[0] = X.sum(), Y.sum(), N
    for c in range(4):
        sel = comp == c
        want[1 + c] = X[sel].sum(), Y[sel].sum(), sel.sum()
    d = _Dev()
    try:
        dpos, drec = d.put(pos), d.put(rec)
        dout = d.put(np.zeros(15, np.float64))
        for _ in range(2):
            rc = L.dsim_signal_noalloc(dpos, drec, N, DSIM_SIGNAL_DSIM3, 0.0, dout, None)
            assert rc == 0, L.dsim_last_error()
            got = d.get(dout, np.zeros(15, np.float64)).reshape(5, 3)
            _close(got, want)
            assert got[0, 2] - got[1:, 2].sum() == (comp > 3).sum() > 0
    finally:
        d.free()


def test_noalloc_signal_rejects_more_spins_than_its_scratch(engine):
    """Rejected on the host before any launch, so the (unused) pointers are
    never dereferenced."""
    from dsim_gb300 import _lib
    L = _lib.native()
    d = _Dev()
    try:
        dummy = d.put(np.zeros(16, np.float32))
        rc = L.dsim_signal_noalloc(dummy, dummy, MAX_SPINS + 1, DSIM_SIGNAL_DSIM3, 0.0, dummy, None)
        assert rc == DSIM_ETOOLARGE
        assert b"limit" in L.dsim_last_error()
    finally:
        d.free()
