"""bench.py on a small scaled workload on the GPU: one JSON line with every
field of the benchmark contract (roofline, CPU baseline, end-to-end figure,
launch count, clocks, the FP32-vs-FP64 and oracle gates), values in range,
and the same `config` as the reference arm prints for that workload."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = ["--scale", "0.15", "--subdomains", "2", "--n-t", "120", "--steps", "3", "--warmup", "3"]


def _line(args, key):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, capture_output=True, text=True,
                       timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [x for x in r.stdout.splitlines() if x.startswith("{") and key in x]
    assert len(lines) == 1, r.stdout[-3000:]
    return json.loads(lines[0])


def test_bench_line_carries_the_contract_fields():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    d = _line(ARGS + ["--no-extra"], '"metric"')
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "roofline", "cpu_baseline", "e2e",
              "gpu_launches", "clocks", "gates"):
        assert k in d, k
    assert d["n_gpus"] == 1 and d["steps"] == 3 and d["warmup"] == 3
    assert d["value"] > 0 and d["unit"] == "DOF-updates/s" and d["higher_is_better"] is True
    assert d["dtype"] == "f32" and d["vs_baseline"] is None
    rf = d["roofline"]
    assert rf["bound"] == "hbm" and rf["unit"] == "GB/s" and 0 < rf["frac"] < 2
    assert abs(rf["frac"] - rf["achieved"] / rf["peak"]) < 1e-9
    assert rf["traffic"] is None or rf["traffic"] > 0
    cb = d["cpu_baseline"]
    assert cb["value"] > 0 and cb["cores"] >= 1 and cb["kind"] == "port" and cb["sample"]
    e = d["e2e"]
    assert 0 < e["value"] and e["h2d_bytes_per_step"] > 0 and e["d2h_bytes_per_step"] > 0
    assert d["gpu_launches"] > 0
    assert {"sm_mhz", "sm_max_mhz", "reasons"} <= set(d["clocks"])
    g = d["gates"]
    assert g["ascan_err_vs_oracle"] <= 1e-4 and g["frame_err_vs_oracle"] <= 1e-4
    assert g["ascan_err_fp64_vs_oracle"] <= 1e-10 and g["frame_times_match"] is True
    ref = _line(ARGS + ["--impl", "reference"], '"impl"')
    assert ref["config"] == d["config"]
