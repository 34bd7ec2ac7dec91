"""bench.py --impl reference (the CPU port of the reference's v6 loop) on a
small scaled workload: one JSON line with the contract's fields, the
reference's own CPU numbers (no GPU, no product code on that path)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--scale", "0.15",
                        "--subdomains", "2", "--steps", "1", "--warmup", "1", "--n-t", "60"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "DOF-updates/s"
    assert d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["config"]["models"] == 3


def test_reference_arm_config_equals_the_product_workload():
    """Both arms print the same `config`: the reference arm builds the
    workload with the oracle's restatements of the reference's generators,
    the product arm with its own; DOFs, stored entries, models, monitors and
    marched samples agree, so the two lines describe one workload."""
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "bristolfe-v2_gb300"))
    import numpy as np
    import bench
    from bfe_gb300 import model
    scale, n_sub, n_t = 0.15, 2, 60
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--scale",
                        str(scale), "--subdomains", str(n_sub), "--steps", "1", "--warmup", "1", "--n-t",
                        str(n_t)], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    ref = json.loads([x for x in r.stdout.splitlines() if x.startswith("{")][0])["config"]
    w = bench.workload(scale)
    w["scale"] = scale
    sides = model.subdomain_sides(n_sub, h=w["h"]) * scale
    subs = [bench._build_subdomain((float(sd), 100 + k)) for k, sd in enumerate(sides)]
    main = model.coupled_water_steel(W=w["W"], H_water=w["H_water"], H_steel=w["H_steel"], h=w["h"],
                                     fc=w["fc"], blob_polygon_pts=w["blob"], array_elements=w["n_src"],
                                     array_pitch=w["pitch"])
    models = [main] + subs
    dt = min(m["dt"] for m in models)
    sig = model.toneburst(np.arange(n_t) * dt, w["fc"], w["cycles"])
    ours = bench.workload_config(w, n_sub, n_t, n_t - int(np.nonzero(sig)[0].min()),
                                 sum(m["K"].shape[0] for m in models),
                                 sum(m["K"].count_nonzero() for m in models), len(models),
                                 sum(len(m["mon_nodes"]) for m in models), 1, scale)
    assert ref == ours


def test_roofline_traffic_record():
    """The step kernel's DRAM traffic that bench.py reports comes from the
    committed capture of the full workload: at its own size it is the
    captured bytes, the other occupancy variant maps to the same record, and
    an unknown kernel reports none."""
    sys.path.insert(0, ROOT)
    import bench
    with open(os.path.join(ROOT, "profiles", "step_kernel_traffic.json")) as f:
        rec = json.load(f)["step_f32_group4<12>"]
    assert bench.profiled_traffic("step_f32_group4<12>", rec["n_dof"]) == rec["dram_bytes_per_launch"]
    assert bench.profiled_traffic("step_f32_group4<10>", rec["n_dof"]) == rec["dram_bytes_per_launch"]
    assert bench.profiled_traffic("no such kernel", 1000) is None
    # the capture's bytes are within 10 % of the algorithmic bytes of that launch
    alg = bench.algorithmic_bytes(72066387, rec["n_dof"], rec["R"], 9, 576, 4)
    assert 0.9 < rec["dram_bytes_per_launch"] / alg < 1.1
