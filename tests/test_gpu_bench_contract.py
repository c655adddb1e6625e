"""bench.py's JSON line on a small workload: every key of the contract
(metric, value, unit, n_gpus, steps, warmup, ms_per_step, higher_is_better,
scaling, vs_baseline, dtype, data, config, e2e with its byte counts,
gpu_launches, clocks, roofline with traffic and peak, cpu_baseline, and the
per-stage roofline) with sane values, for the plain and the precision form."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _line(*args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    return json.loads(lines[0])


@pytest.mark.parametrize("args", [
    ("--workload", "spheres3d_64", "--steps", "3", "--warmup", "3", "--forms", "0"),
    ("--workload", "spheres3d_64", "--precision", "mixed", "--sweep-form", "fused", "--steps", "3", "--warmup", "3",
     "--forms", "0", "--no-cpu-baseline"),
])
def test_bench_line_contract(args):
    d = _line(*args)
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "e2e", "gpu_launches", "clocks", "roofline"):
        assert k in d, k
    assert d["n_gpus"] == 1 and d["steps"] == 3 and d["warmup"] == 3
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["higher_is_better"] is True
    assert d["config"]["workload"].startswith("3D ibm3 unit cube 64^3")
    e2e = d["e2e"]
    assert e2e["value"] > 0 and e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] > 0
    assert e2e["value"] < d["value"]  # host copies inside the timed region
    assert d["gpu_launches"] > 0
    assert "sm_mhz" in d["clocks"] and "reasons" in d["clocks"]
    rf = d["roofline"]
    assert rf["bound"] in ("hbm", "tensor") and rf["unit"] == "GB/s"
    assert rf["achieved"] > 0 and rf["peak"] > 0 and abs(rf["frac"] - rf["achieved"] / rf["peak"]) < 1e-9
    assert "traffic" in rf
    st = d["stages"]
    stages = ("predictor", "rhs", "sor", "projection_boundary")
    assert all(st[k]["ms_per_step"] > 0 and st[k]["achieved_gbs"] > 0 for k in stages)
    assert abs(sum(st[k]["ms_per_step"] for k in stages) - d["ms_per_step"]) <= 0.01 * d["ms_per_step"] + 0.01
    assert st["peak_gbs"] == rf["peak"]
    if "--precision" in args:
        assert d["dtype"] == "f32+f64" and rf["kernel"] == "k_sor_fused3"
        assert rf["cell_updates_per_launch"] == 64 ** 3  # one launch per full sweep
    else:
        # the plain 3D case walks its cell lists (pf_sor_list.cu); its FP64 rate
        # is counted on the reference's 14 flops per update ("effective")
        assert d["dtype"] == "f64" and rf["kernel"] == "k_sor_list3"
        assert rf["cell_updates_per_launch"] == 64 ** 3 / 2  # one launch per colour
        assert rf["fp64_alu"]["counting"].startswith("effective") and rf["fp64_alu"]["frac"] > 0
        cb = d["cpu_baseline"]
        assert cb["kind"] == "port" and cb["value"] > 0 and cb["cores"] >= 1 and cb["sample"]
