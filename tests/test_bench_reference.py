"""bench.py's reference arm: the reference algorithm (the FP64 oracle
restatement of origin/GoldenC/src/main.c with the fan tracer) timed on the
host cores, printing the same metric, unit and config as the GPU arm.

Under torchrun only rank 0 runs it; every other rank exits 0 without work and
prints nothing."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                           "--steps", "1", "--warmup", "1"],
                          cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)


def test_reference_arm_line(oracle):
    sys.path.insert(0, ROOT)
    import bench

    p = _run({"RANK": "0", "WORLD_SIZE": "1"})
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    out = json.loads(lines[0])
    assert out["impl"] == "reference"
    assert out["metric"] == bench.METRIC and out["unit"] == bench.UNIT
    assert out["higher_is_better"] is True
    assert out["steps"] == 1 and out["warmup"] == 1 and out["n_gpus"] == 1
    assert out["value"] > 0
    assert out["config"]["workload"] == bench.WORKLOAD
    cb = out["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["unit"] == bench.UNIT and cb["sample"]
    assert cb["value"] == out["value"]
    e2e = out["e2e"]
    assert e2e == {"value": out["value"], "unit": bench.UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_do_no_work():
    p = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert p.returncode == 0, p.stderr[-2000:]
    assert p.stdout.strip() == ""
