"""bench.py's reference arm runs on the host alone (the CPU restatement of the step): its JSON line
carries the contract's keys, the same metric and unit as the GPU arm, impl = reference, a
cpu_baseline describing the run and an e2e object without host-device copies."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "small", "--steps", "3",
                        "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    import bench
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "e2e", "cpu_baseline"):
        assert k in d, k
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == "steps/s"
    assert d["steps"] == 3 and d["warmup"] == 3 and d["value"] > 0 and d["higher_is_better"] is True
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"] and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["config"]["workload"] == "hydrogen_velocity_small"


def test_reference_arm_batch_and_adjoint():
    """The batch workload's reference arm times the restatement on a sample of the same seeded
    problems (batch steps/s); the adjoint has no reference counterpart and says so."""
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "batch", "--batch-size", "12",
                        "--steps", "2", "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
    assert d["impl"] == "reference" and d["unit"] == "batch steps/s" and d["value"] > 0
    assert d["config"]["problems"] == 12 and d["e2e"]["h2d_bytes_per_step"] == 0
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "adjoint"], cwd=ROOT,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    d = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
    assert d["impl"] == "reference" and "unavailable" in d
