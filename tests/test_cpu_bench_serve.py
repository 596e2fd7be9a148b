"""bench.py's serving stream on the host, against a stand-in for the request
loop that records what it is given: every job is submitted once, in order,
with its own arrays and form; jobs generated ahead on host threads are the
jobs a plain list would give; signals come back for the kept jobs only; the
Poisson gaps follow the seed.  No GPU call is made."""
import os
import sys
import time

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class _Sub:
    def __init__(self, kind):
        self.kind, self.handle = kind, object()


class _FakeServer:
    made = []

    def __init__(self, spin_capacity, job_capacity, hbm_cap):
        self.cap, self.jobs, self.hbm = spin_capacity, job_capacity, hbm_cap
        self.subs, self.sub_list, self.t0 = [], [], None
        _FakeServer.made.append(self)

    def add_mesh(self, h):
        self.sub_list.append(("mesh", h))
        return len(self.sub_list) - 1

    def add_cyl(self, h):
        self.sub_list.append(("cyl", h))
        return len(self.sub_list) - 1

    def configure(self, **kw):
        self.cfg = kw

    def start(self):
        self.t0 = time.perf_counter()

    def submit(self, sid, pos, comp, fiber, grads, **kw):
        t = time.perf_counter() - self.t0
        self.subs.append((sid, pos.copy(), comp.copy(), grads.copy(), kw, t))
        return len(self.subs) - 1

    def drain(self):
        pass

    def stats(self):
        return {"max_inflight": 3.0, "errors": 0.0, "hbm_peak": 5e9}

    def stop(self):
        pass

    def poll(self, t):
        sid, pos, comp, grads, kw, ts = self.subs[t]
        sig = np.full((len(grads), 5, 3), float(t))
        return True, sig, np.array([ts, ts + 0.001, ts + 0.01 + 0.001 * t])

    def close(self):
        pass


def _job(subs, k):
    rng = np.random.default_rng([5, k])
    n = int(rng.integers(32, 200))
    return {"sub": subs[k % 2], "pos": rng.uniform(-1, 1, 3 * n).astype(np.float32),
            "comp": np.zeros(n, np.uint8), "fiber": np.zeros(n, np.uint32), "n": n, "steps": 10 + k,
            "grads": rng.normal(size=(3, 3)).astype(np.float32), "dt": np.float32(0.01),
            "step_sd": np.zeros(4, np.float32), "T2": np.zeros(4, np.float32), "phase_constant": 1.0, "seed": k,
            "permeability": 0.0, "delta": 1.0, "Delta": 2.0, "inner": 1.0}


@pytest.fixture
def bench(monkeypatch):
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench as B
    from dsim_gb300 import engine
    monkeypatch.setattr(engine, "Server", _FakeServer)
    _FakeServer.made.clear()
    return B


@pytest.mark.parametrize("ahead", [0, 5])
def test_stream_submits_every_job_once_in_order(bench, ahead):
    subs = [_Sub("mesh"), _Sub("cyl")]
    n = 23
    jobs = [_job(subs, k) for k in range(n)]
    keep = {3, 11, 20}
    o, sigs = bench.serve_stream(subs, lambda k: _job(subs, k), n, {"chunk": 20, "occupancy": 4}, 400.0, "bar",
                                 1 << 20, ahead=ahead, keep=keep)
    srv = _FakeServer.made[-1]
    assert srv.cap == 1 << 20 and srv.jobs == n and srv.hbm == 150e9
    assert len(srv.subs) == n
    for k, (sid, pos, comp, grads, kw, _) in enumerate(srv.subs):
        j = jobs[k]
        assert srv.sub_list[sid][0] == j["sub"].kind
        assert np.array_equal(pos, j["pos"]) and np.array_equal(grads, j["grads"])
        assert kw["steps"] == j["steps"] and kw["seed"] == k
        assert kw.get("local") is True and not kw.get("precise")     # the error-bar form: cell-local
    assert set(sigs) == keep
    for k in keep:
        assert sigs[k].shape == (3, 5, 3) and np.all(sigs[k] == k)
    assert o["errors"] == 0 and o["max_jobs_in_flight"] == 3 and o["hbm_peak_GB"] == 5.0
    work = sum(j["n"] * j["steps"] for j in jobs)
    assert o["spin_steps_per_s"] > 0 and abs(o["spin_steps_per_s"] * o["wall_s"] - work) < 1e-6 * work
    # arrivals follow the seeded exponential gaps (400 jobs/s: about 2.5 ms apart)
    t = np.array([s[5] for s in srv.subs])
    want = np.cumsum(np.random.default_rng(3).exponential(1 / 400.0, n))
    assert np.all(t >= want - 1e-3)


def test_served_mix_keeps_list_order(bench):
    subs = [_Sub("mesh"), _Sub("cyl")]
    mix = [_job(subs, k) for k in range(9)]
    o, sigs = bench.run_served_mix(subs, mix, {"chunk": 20, "occupancy": 4}, 1000.0, form="fp32")
    assert [float(s[0, 0, 0]) for s in sigs] == list(range(9))
    srv = _FakeServer.made[-1]
    assert all("local" not in s[4] and "precise" not in s[4] for s in srv.subs)
    cap = max(sum((j["n"] + 31) // 32 * 32 for j in mix) // 2, max((j["n"] + 31) // 32 * 32 for j in mix))
    assert srv.cap == cap
