"""CPU: the benchmark's reference arm (`bench.py --impl reference`), which
needs no GPU: one JSON line with the fields the harness reads, its step
defaults, the zero-copy e2e object, and the rank and workload rules."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SMALL = "r2c_c2r_64x64x64_f64_x"


def run_bench(*args, env_extra=None):
    env = dict(os.environ)
    env.update(env_extra or {})
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    return [json.loads(ln) for ln in lines]


def test_reference_arm_line_and_defaults():
    import bench
    (out,) = run_bench("--impl", "reference", "--workload", SMALL)
    assert out["impl"] == "reference"
    assert out["metric"] == bench.METRIC
    assert out["unit"] == "GPts/s" and out["higher_is_better"] is True
    assert out["steps"] == 20 and out["warmup"] == 3  # whole CPU round trips by default
    assert out["value"] > 0 and out["ms_per_step"] > 0
    assert out["value"] == pytest.approx(64 ** 3 / (out["ms_per_step"] * 1e-3) / 1e9, rel=1e-2)
    cb = out["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == out["value"] and cb["sample"]
    e2e = out["e2e"]
    assert e2e["value"] == out["value"] and e2e["unit"] == out["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert out["config"]["name"] == SMALL and out["dtype"] == "f64"


def test_reference_arm_keeps_the_steps_it_is_given_and_at_least_three_warmups():
    (out,) = run_bench("--impl", "reference", "--workload", SMALL, "--steps", "2", "--warmup", "1")
    assert out["steps"] == 2 and out["warmup"] == 3


def test_reference_arm_prints_nothing_on_other_ranks():
    outs = run_bench("--impl", "reference", "--workload", SMALL,
                     env_extra={"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert outs == []


def test_reference_arm_of_a_workload_without_a_cpu_run_says_so():
    import bench
    (out,) = run_bench("--impl", "reference", "--workload", bench.BATCH_WORKLOAD)
    assert out["impl"] == "reference" and "unavailable" in out
