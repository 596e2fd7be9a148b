"""bench.py --impl reference on the host alone: the oracle builds the mesh
arrays and grid and times the reference's CPU step on a sample; the line
carries the contract's keys (impl, cpu_baseline, e2e with no copies)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_runs_on_host_cores(engine):
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--axons", "12",
                          "--spins", "8192", "--steps", "1", "--warmup", "3", "--cpu-seconds", "0.5"],
                         capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    r = json.loads(out.stdout.strip().splitlines()[-1])
    assert r["impl"] == "reference" and r["unit"] == "spin-steps/s" and r["value"] > 0
    assert r["higher_is_better"] is True and r["n_gpus"] == 1
    cb = r["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == r["value"]
    assert "oracle" in cb["sample"]
    e = r["e2e"]
    assert e["value"] == r["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
