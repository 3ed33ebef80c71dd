"""bench.py's reference arm: the reference algorithm (the FP64 oracle
restatement of origin/GoldenC/src/main.c with the fan tracer) timed on the
host cores, printing the same metric, unit and config as the GPU arm.

Under torchrun only rank 0 runs it; every other rank exits 0 without work and
prints nothing.

Also the GPU arm's GoldenC side sample (GoldenC at its own geometry beside the
drop-in entry points), driven here by an oracle-backed stand-in library: its
fields, and an error field rather than an exception when the library fails."""
import json
import os
import subprocess
import sys

import numpy as np

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


class _OracleDropin:
    """GoldenC's drop-in entry points answered by the FP64 oracle, so that the
    bench's GoldenC sample can be exercised without a GPU."""

    def __init__(self, oracle):
        self.o = oracle

    def A(self, proj, img):
        proj[...] = self.o.gc_A(img)

    def minimize_in_IMAGE_variable(self, out, g, f, v, alpha, epsilon, it):
        out[...] = self.o.image_step(None, g, f, v, alpha, epsilon, it)[0]

    def minimize_in_EDGE_variable(self, out, f, v, alpha, beta, epsilon, it):
        out[...] = self.o.edge_step(f, v, alpha, beta, epsilon, it)[0]

    def goldnc_status(self):
        return 0


def test_goldnc_sample_fields_and_errors(oracle):
    import types

    sys.path.insert(0, ROOT)
    import bench
    import medimage_gb300.phantom as phantom

    mg = types.SimpleNamespace(lib=lambda: _OracleDropin(oracle), phantom=phantom)
    out = bench.run_goldnc_native(mg, reps=1)
    assert "error" not in out, out
    assert out["goldnc_cpu"] == {"cores": 1, "kind": "port"}
    assert out["engine_dropin_s"] > 0 and out["goldnc_cpu_s"] > 0 and out["status"] == 0
    assert out["rel_l2_f"] == 0.0 and out["rel_l2_v"] == 0.0  # the stand-in is the oracle itself

    def broken():
        raise OSError("library missing")

    bad = bench.run_goldnc_native(types.SimpleNamespace(lib=broken, phantom=phantom), reps=1)
    assert bad == {"error": "OSError: library missing"}


def test_parity_block_fields(oracle):
    """bench.py's C2 parity block, assembled on a small slice with the oracle
    standing in for both engine forms (so every rel-L2 is 0 up to the order of
    the oracle's own OpenMP sums, and every exit trace agrees): the background FP64 solve, the fields, the units."""
    import types

    sys.path.insert(0, ROOT)
    import bench
    import medimage_gb300.phantom as phantom
    from medimage_gb300 import configs
    from medimage_gb300.engine import FanGeometry

    spec = configs.SliceSpec(FanGeometry.covering(48, 2.0, 60, 80), 1e4, 5, 2, 2)
    fan = oracle.fan_from_engine(spec.geom)
    ph = phantom.ellipse_phantom(48, seed=5, n_random=2)
    sino = phantom.poisson_sinogram(oracle.fan_A(fan, ph.astype(np.float64)), 1e4, 6)
    ora = bench.OracleSolve(spec, sino, 2)
    fo, vo, tr = oracle.solve(fan, sino.astype(np.float64), 1000.0, 0.002, 1e-4, 2, 10, 10)
    trace = [(o, s, k, e, ()) for (o, s, k, _, e) in tr]
    form = {"fp": oracle.fan_A(fan, ph.astype(np.float64)), "bp": oracle.fan_AT(fan, sino.astype(np.float64)),
            "f": fo, "v": vo, "trace": trace, "segments": oracle.fan_segments(fan)}
    mg = types.SimpleNamespace(phantom=phantom)
    out = bench.finish_parity(mg, spec, {"fp64_alpha": form, "fp32_alpha": form}, ora, ph, sino)
    assert "error" not in out, out
    assert out["oracle_solve_s"] > 0 and out["oracle_threads"] == 2
    assert out["segments_fp64_oracle"] == form["segments"]
    for name in ("fp64_alpha", "fp32_alpha"):
        ent = out[name]
        assert ent["forward_rel_l2"] == 0.0 and ent["back_rel_l2"] == 0.0
        # the background solve runs on 2 threads, the stand-in's on all:
        # OpenMP reductions in another order
        assert ent["f_rel_l2"] <= 1e-12 and ent["v_rel_l2"] <= 1e-12
        assert abs(ent["psnr_minus_fp64_db"]) <= 1e-3 and ent["exit_branches_identical"] is True
    json.dumps(out)
