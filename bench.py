"""Benchmark of the explicit time-marching path on one GB300 (or N replicas).

Headline: FP32 batched time marching of 64 sources (64 right-hand sides) on
the coupled water/steel model - 60 x 30 mm at 0.05 mm (1.44M triangles),
ASI2D2 interface, quadratic absorbing layers, seeded void, 64-element array on
the water surface - together with 32 steel scatterer sub-domain models of
50k-400k DOF (absorbers, seeded voids) in one multi-model plan, over 6,000
samples, replayed as CUDA graphs. One bench step = one full march of all
sources of all models. Also measured in the same run: the plain FP64 form on
the same models (one source), the max-normalised A-scan error of the FP32
batched result against that FP64 run, the coupled model alone, the step
kernel's roofline, the end-to-end call through the C ABI with host buffers,
and the FP64 CPU restatement of the reference's time loop on the host cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "bristolfe-v2_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "DOF-updates/s & HBM GB/s: FP32 batched vs plain FP64 GPU at ≤1e-4 A-scan err"
UNIT = "DOF-updates/s"

WORKLOAD = dict(W=60e-3, H_water=20e-3, H_steel=10e-3, h=0.05e-3, fc=5e6, cycles=5,
                n_t=6000, n_src=64, pitch=0.6e-3, blob_radius=1.5e-3, seed=0)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=float, default=1.0,
                    help="shrink the model size (testing only; 1.0 = the benchmark model)")
    ap.add_argument("--n-t", type=int, default=None)
    ap.add_argument("--sources", type=int, default=None,
                    help="array elements = right-hand sides (default 64, the benchmark; at most 64)")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the extra sections (C0 plate, FMC, assembly, 3D, adjoint); runs with "
                         "more than one GPU always skip them")
    ap.add_argument("--subdomains", type=int, default=32,
                    help="steel sub-domain models marched with the coupled model (32 = benchmark)")
    ap.add_argument("--only", choices=["adjoint", "c1"], default=None,
                    help="run one extra section alone and print its JSON (profiling); --n-t sets its "
                         "samples, finite-difference checks are skipped")
    return ap.parse_args()


def blob_polygon(radius, centre, seed, n_harm=8, amp_max=0.2, n_pts=128):
    """Seeded smooth random void: r(a) = R (1 + sum_k A_k sin(k a + phi_k)) /
    (1 + sum A_k / 2), A_k ~ U(0, amp_max), k = 1..n_harm."""
    rng = np.random.default_rng(seed)
    A = rng.uniform(0.0, amp_max, n_harm)
    phi = rng.uniform(0.0, 2 * np.pi, n_harm)
    a = np.linspace(0, 2 * np.pi, n_pts, endpoint=False)
    k = np.arange(1, n_harm + 1)
    r = radius * (1 + (A[None, :] * np.sin(a[:, None] * k[None, :] + phi[None, :])).sum(1)) / (1 + A.sum() / 2)
    return np.column_stack([r * np.cos(a), r * np.sin(a)]) + np.asarray(centre)


def workload(scale):
    w = dict(WORKLOAD)
    if scale != 1.0:
        w["W"] *= scale
        w["H_water"] *= scale
        w["H_steel"] *= scale
        w["pitch"] *= scale
        w["blob_radius"] *= scale
    w["blob"] = blob_polygon(w["blob_radius"], (w["W"] / 2, w["H_steel"] / 2), w["seed"])
    return w


class ClockSampler:
    """nvidia-smi SM clock / throttle-reason sampling during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


KERNEL_NAMES = {
    0: "step_batched<float,2> (slice-staged rows)",
    9: "step_f32_group2<2,1,1>", 10: "step_f32_group2<2,2,1>", 11: "step_f32_group2<2,4,1>",
    12: "step_f32_group2<2,1,4>", 13: "step_f32_group2<2,1,6>", 14: "step_f32_group2<2,1,8>",
    20: "step_f32_group4<12>", 22: "step_f32_group4<10>",
}


def profiled_traffic(kernel, n_dof):
    """DRAM bytes per launch of `kernel` from the committed ncu summary
    (profiles/step_kernel_traffic.json), scaled to n_dof rows, or None."""
    p = os.path.join(ROOT, "profiles", "step_kernel_traffic.json")
    try:
        with open(p) as f:
            d = json.load(f)
    except (OSError, ValueError):
        return None
    rec = d.get(kernel) or d.get(d.get("_same_traffic", {}).get(kernel, ""))
    if not rec:
        return None
    return rec["dram_bytes_per_launch"] * n_dof / rec["n_dof"]


def algorithmic_bytes(nnz, n, R, p, q, b):
    """Bytes one time step must move (per launch of the step kernel):
    operator values + int32 columns, row pointers, two per-row coefficient
    vectors, read u_n, read u_{n-1}, write u_{n+1} per RHS, forcing and
    monitor values."""
    return nnz * (b + 4) + 4 * (n + 1) + 2 * n * b + 3 * R * n * b + R * (p + q) * b


SUB_MONITORS = 16      # monitored nodes per steel sub-domain model
L2_BYTES = 126 * 2 ** 20   # GB300 L2


def workload_config(w, n_sub, n_t, steps_per_march, n_dof, nnz, n_models, n_mon, world, scale):
    """The `config` object of both arms' JSON lines: the workload itself
    (the same dict from `--impl ours` and `--impl reference` at a given N);
    how an arm ran it is reported outside `config`."""
    R = w["n_src"]
    return {"workload": "batched multi-source and multi-model: coupled water/steel "
                        "60x30 mm at 0.05 mm (1.44M triangles, ASI2D2 interface, quadratic "
                        "absorbers, void blob) with a %d-element array, plus %d steel "
                        "scatterer sub-domain models of 50k-400k DOF (absorbers, void), "
                        "%d sources as %d RHS, %d samples" % (R, n_sub, R, R, n_t),
            "n_dof": int(n_dof), "nnz_K": int(nnz), "models": int(n_models), "sources": R,
            "monitors": int(n_mon), "samples": int(n_t), "steps_marched_per_source": int(steps_per_march),
            "l2": ("inputs larger than L2" if 3 * R * n_dof * 4 > L2_BYTES else "inputs within L2") +
                  " (FP32 state %.0f MB per time step)" % (3 * R * n_dof * 4 / 1e6),
            "parallelism": ("one GPU" if world == 1 else
                            "%d ranks, models split by cost, no data-path collective" % world),
            "scale": scale}


def _build_subdomain(args):
    """Worker: one steel sub-domain model (runs in a spawned process)."""
    import bfe_gb300.model as model
    side, seed = args
    m = model.steel_subdomain(side, seed=seed, n_mon=SUB_MONITORS)
    return {k: m[k] for k in ("K", "C", "M", "gl", "dt", "src_nodes", "mon_nodes")}


def build_workload(w, n_sub):
    """Coupled FMC model plus n_sub steel sub-domain models (built in a spawn
    pool before any GPU work)."""
    from concurrent.futures import ProcessPoolExecutor
    import multiprocessing as mp
    from bfe_gb300 import model
    sides = model.subdomain_sides(n_sub, h=w["h"]) * (1.0 if w.get("scale", 1.0) == 1.0 else w["scale"])
    subs = []
    if n_sub:
        with ProcessPoolExecutor(max_workers=min(n_sub, os.cpu_count() or 4),
                                 mp_context=mp.get_context("spawn")) as ex:
            subs = list(ex.map(_build_subdomain, [(float(sd), 100 + k) for k, sd in enumerate(sides)]))
    main = model.coupled_water_steel(W=w["W"], H_water=w["H_water"], H_steel=w["H_steel"], h=w["h"],
                                     fc=w["fc"], blob_polygon_pts=w["blob"],
                                     array_elements=w["n_src"], array_pitch=w["pitch"])
    return main, subs


def _model_costs(models, R):
    """Bytes one FP32 time step of each model moves with R sources (the
    sharding weights)."""
    return [algorithmic_bytes(m["K"].nnz, m["K"].shape[0], R, 1, len(m["mon_nodes"]), 4) for m in models]


def _dof_groups(models, offs):
    """Row groups of a joined operator for per-group max-normalised errors:
    each model's fluid (pressure) rows and its solid (displacement) rows."""
    from bfe_gb300.solver import dof_maps_from_lookup
    groups = []
    for k, m in enumerate(models):
        _, typ = dof_maps_from_lookup(m["gl"], m["K"].shape[0])
        for fluid in (True, False):
            rows = np.nonzero((typ == 4) == fluid)[0]
            if rows.size:
                groups.append(rows + offs[k])
    return groups


def _max_err(a, b, groups):
    """Largest per-group max-normalised difference (a against b). A group
    whose reference peak is below 1e-20 of the largest group's peak is left
    out: the wave has not reached it yet, and its FP64 values are round-off
    leakage (1e-70 and below) that FP32 cannot represent."""
    peaks = [float(np.abs(b[g]).max()) for g in groups]
    top = max(peaks, default=0.0)
    out = 0.0
    for g, ref in zip(groups, peaks):
        if ref > 0 and ref >= 1e-20 * top:
            out = max(out, float(np.abs(a[g] - b[g]).max() / ref))
    return out


def run_ours(args):
    from bfe_gb300 import model, shard
    w = workload(args.scale)
    w["scale"] = args.scale
    if args.sources:
        if not 1 <= args.sources <= 64:
            raise SystemExit("--sources must be between 1 and 64")
        w["n_src"] = args.sources
    n_t = args.n_t or w["n_t"]
    t0 = time.perf_counter()
    main, subs = build_workload(w, args.subdomains)
    t_build = time.perf_counter() - t0

    import torch
    import bfe_gb300
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    bfe_gb300.load()
    models = [main] + subs
    dt = min(m["dt"] for m in models)
    t = np.arange(n_t) * dt
    sig = model.toneburst(t, w["fc"], w["cycles"])
    R_all = w["n_src"]
    # this rank's share: models by cost (all sources), or sources when ranks
    # outnumber models; one rank marches everything
    mine, (s_lo, s_hi) = shard.rank_share(_model_costs(models, R_all), R_all, world, rank)
    R = s_hi - s_lo
    sel_models = [models[k] for k in mine]
    t0 = time.perf_counter()
    plan32, offs = bfe_gb300.Plan.multi([(m["K"], m["C"], m["M"], m["gl"]) for m in sel_models], dt,
                                        bfe_gb300.VEL_CURRENT, "single")
    t_plan = time.perf_counter() - t0
    n = plan32.n
    nnz = sum(m["K"].nnz for m in sel_models)

    def src_dofs(k, m, r):
        """1-based DOFs of source r in model k: array element r of the coupled
        model (pressure), source r of a sub-domain model (displacement)."""
        return model.global_indices(m["gl"], m["src_nodes"][r], 4 if k == 0 else 2)

    srcs = [np.concatenate([src_dofs(k, m, r) + offs[j] for j, (k, m) in enumerate(zip(mine, sel_models))])
            for r in range(s_lo, s_hi)]
    mon_parts = [model.global_indices(m["gl"], m["mon_nodes"], 4 if k == 0 else 2) + offs[j]
                 for j, (k, m) in enumerate(zip(mine, sel_models))]
    mons = np.concatenate(mon_parts)
    mon_model = np.concatenate([np.full(p.size, j) for j, p in enumerate(mon_parts)])
    q = mons.size
    p_max = max(s_.size for s_ in srcs)
    frc_dof = np.concatenate([s_ - 1 for s_ in srcs])
    frc_rhs = np.concatenate([np.full(s_.size, r) for r, s_ in enumerate(srcs)])
    frc_sig = np.zeros(frc_dof.size, np.int64)
    stream = torch.cuda.Stream()
    d_sig = torch.tensor(sig, dtype=torch.float64, device="cuda").reshape(n_t, 1)
    d_hist = torch.zeros((R, n_t, q), dtype=torch.float64, device="cuda")
    ti0 = int(np.nonzero(sig)[0].min())
    steps_per_march = n_t - ti0

    def march32(plan=plan32, hist=d_hist, dofs=frc_dof, rhs=frc_rhs, fsig=frc_sig, mon=mons, r=R):
        with torch.cuda.stream(stream):
            hist.zero_()
        plan.run_device(r, n_t, ti0, dofs, rhs, fsig, None, d_sig, mon - 1, hist, stream.cuda_stream)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def reduce(x, op):
        if dist is None:
            return x
        tt = torch.tensor([float(x)], dtype=torch.float64, device="cuda")
        dist.all_reduce(tt, op=op)
        return float(tt.item())

    for _ in range(args.warmup):
        march32()
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        barrier()
        ev0.record(stream)
        for _ in range(args.steps):
            march32()
        ev1.record(stream)
        barrier()
    ms_total = ev0.elapsed_time(ev1)
    MAX = dist.ReduceOp.MAX if dist is not None else None
    SUM = dist.ReduceOp.SUM if dist is not None else None
    ms_total = reduce(ms_total, MAX)                          # the slowest rank
    ms_step = ms_total / args.steps
    # distinct work of all ranks: each rank's sources x DOFs x steps
    dof_updates = reduce(float(R * n * steps_per_march), SUM)
    n_all = sum(m["K"].shape[0] for m in models)
    st32 = plan32.stats()
    launches = args.steps * (st32["step_launches"] + st32["aux_launches"])
    value = dof_updates / (ms_step * 1e-3)
    h32 = d_hist.cpu().numpy()                                # (R, n_t, q)
    local_ascans = {k: h32[:, :, mon_model == j] for j, k in enumerate(mine)}

    # per-kernel timing pass (CUDA events around every launch, same stream)
    plan32.set_timing(True)
    march32()
    torch.cuda.synchronize()
    stk = plan32.stats()
    plan32.set_timing(False)
    step_avg_ms = stk["step_ms"] / max(stk["step_launches"], 1)
    aux_avg_ms = stk["aux_ms"] / max(stk["aux_launches"], 1)
    kname = KERNEL_NAMES.get(stk["variant"], "variant %d" % stk["variant"])
    bytes_step = algorithmic_bytes(nnz, n, R, p_max, q, 4)
    peak, peak_kind = measured_peak_hbm()
    achieved = bytes_step / (step_avg_ms * 1e-3) / 1e9

    # end to end through the C ABI with host buffers (H2D signals, D2H A-scans)
    barrier()
    th0 = time.perf_counter()
    plan32.run_batched(t, srcs, sig, mons)
    e2e_s = reduce(time.perf_counter() - th0, MAX)
    e2e_value = dof_updates / e2e_s
    h2d = reduce(8 * n_t * R + 8 * (p_max * R + q), SUM)
    d2h = reduce(8 * q * n_t * R, SUM)

    # A-scans of every model and source on rank 0 (outside the timed region)
    if dist is not None:
        ascans = shard.gather_model_ascans(local_ascans, s_lo, R_all, dist)
    else:
        ascans = local_ascans
    if rank == 0:
        assert sorted(ascans) == list(range(len(models))), "A-scans of some models are missing"

    extra, gates, fp64 = {}, {}, None
    if world == 1:
        fp64, gates = fp64_and_oracle_sections(torch, bfe_gb300, model, models, plan32, offs, srcs, mons,
                                               mon_model, h32, d_sig, stream, t, sig, dt, ti0, nnz, value,
                                               args.no_extra)
        # the extra sections run in one-GPU runs only: under torchrun the
        # other ranks would hold their GPUs idle in the final barrier meanwhile
        if not args.no_extra:
            extra.update(subsection_rooflines(torch, bfe_gb300, models, offs, frc_dof, frc_rhs, frc_sig,
                                              mons, march32, R, n_t, ti0, peak, dt, stream))
            extra["plate_c0"] = plate_c0_section(bfe_gb300, model)
            extra["coupled_c1"] = coupled_c1_section(torch, bfe_gb300, model, main, peak)
            extra["fmc_c2a"] = fmc_section(torch, bfe_gb300, d_hist, R, n_t, q, mon_parts[0].size, sig, stream)
            extra["assembly_c1"] = assembly_section(torch, bfe_gb300, model, main)
            extra["hex3d_c3"] = hex3d_section(torch, bfe_gb300, model)
            extra["adjoint_c4"] = adjoint_section(torch, bfe_gb300, model)
    result = None
    if rank == 0:
        cpu = gates.pop("_cpu_baseline", None)
        n_sub = len(subs)
        result = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": workload_config(w, n_sub, n_t, steps_per_march, n_all,
                                      sum(m["K"].count_nonzero() for m in models), len(models),
                                      sum(len(m["mon_nodes"]) for m in models), world, args.scale),
            "run": {"kernel_path": "FP32 batched, CUDA graph",
                    "rank0_share": {"models": len(mine), "n_dof": n, "sources": [s_lo, s_hi],
                                    "state_mb_per_step": 3 * R * n * 4 / 1e6}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": profiled_traffic(kname, n),
                         "kernel": kname, "variant": stk["variant"], "bytes_per_launch": bytes_step,
                         "avg_launch_ms": step_avg_ms, "peak_source": peak_kind,
                         "interface_kernel_avg_ms": aux_avg_ms},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "s_per_step": e2e_s},
            "gpu_launches": launches,
            "clocks": clocks.summary(),
            "setup_s": {"model_build": t_build, "plans": t_plan},
            "cpu_baseline": cpu,
        }
        result.update(extra)
        # the headline gates last, so that a tail of the line keeps them
        if fp64 is not None:
            result["fp64_plain"] = fp64
        result["gates"] = gates
        print(json.dumps(result), flush=True)
    plan32.close()
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return result


def fp64_and_oracle_sections(torch, bfe_gb300, model, models, plan32, offs, srcs, mons, mon_model, h32,
                             d_sig, stream, t, sig, dt, ti0, nnz, value, quick=False):
    """One-GPU checks of the headline result (the middle source r):
      - the plain FP64 GPU form on the same models (its DOF-updates/s and the
        FP32 batched speed-up over it, the metric's comparison);
      - the FP32 batched A-scans against that FP64 run over all samples;
      - the FP64 C port of the reference's v6 loop on the joined operator
        (the CPU baseline, timed on a bounded prefix of the march) as the
        oracle: the FP32 batched and the FP64 A-scans, and FP32 field frames
        of the same source (one-source run on the FP32 plan), against it.
    Errors are max-normalised per model and per kind of DOF (pressure,
    displacement). Returns (fp64 dict, gates dict with the CPU baseline
    under "_cpu_baseline")."""
    R, n_t, q = h32.shape
    n = plan32.n
    r_mid = R // 2
    plan64, _ = bfe_gb300.Plan.multi([(m["K"], m["C"], m["M"], None) for m in models], dt,
                                     bfe_gb300.VEL_CURRENT, "double")
    d_hist64 = torch.zeros((1, n_t, q), dtype=torch.float64, device="cuda")
    src = srcs[r_mid]

    def march64():
        with torch.cuda.stream(stream):
            d_hist64.zero_()
        plan64.run_device(1, n_t, ti0, src - 1, np.zeros(src.size, np.int64), np.zeros(src.size, np.int64),
                          None, d_sig, mons - 1, d_hist64, stream.cuda_stream)
    march64()
    torch.cuda.synchronize()
    k64 = 2
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(k64):
        march64()
    e1.record(stream)
    torch.cuda.synchronize()
    ms64 = e0.elapsed_time(e1) / k64
    value64 = n * (n_t - ti0) / (ms64 * 1e-3)
    plan64.set_timing(True)
    march64()
    torch.cuda.synchronize()
    st64 = plan64.stats()
    plan64.set_timing(False)
    step64_ms = st64["step_ms"] / max(st64["step_launches"], 1)
    aux64_ms = st64["aux_ms"] / max(st64["aux_launches"], 1)
    bytes64 = algorithmic_bytes(nnz, n, 1, src.size, q, 8)
    h64 = d_hist64.cpu().numpy()[0]                       # (n_t, q)
    plan64.close()
    mon_groups = [np.nonzero(mon_model == k)[0] for k in range(len(models))]
    err_fp64 = _max_err(h32[r_mid].T, h64.T, mon_groups)
    fp64 = {"value": value64, "unit": UNIT, "ms_per_march": ms64, "step_kernel_ms": step64_ms,
            "interface_kernel_ms": aux64_ms, "step_kernel_gbs": bytes64 / (step64_ms * 1e-3) / 1e9}

    # the oracle: FP64 C port on the joined operator, a bounded prefix
    import scipy.sparse as sp
    Kj = sp.block_diag([m["K"] for m in models], format="csr")
    Cj = sp.block_diag([m["C"] for m in models], format="csr")
    Mj = sp.block_diag([m["M"] for m in models], format="csr")
    cpu, (ho, fo, fto, steps, every) = cpu_baseline(Kj, Cj, Mj, dt, t, src, sig, mons,
                                                    target_s=4.0 if quick else 10.0)
    cpu["sample"] += ", all %d models joined in one operator" % len(models)
    err32_orc = _max_err(h32[r_mid][:steps].T, ho, mon_groups)
    err64_orc = _max_err(h64[:steps].T, ho, mon_groups)
    # FP32 frames of the same source from a one-source run on the FP32 plan
    _, f32, ft32 = plan32.run(t[:steps], src, sig[:steps], mons, every, True)
    groups = _dof_groups(models, offs)
    frame_err = _max_err(f32, fo, groups)
    gates = {"speedup_fp32_batched_vs_fp64_plain": value / value64,
             "ascan_err_vs_fp64": err_fp64,
             "ascan_err_vs_oracle": err32_orc, "ascan_err_fp64_vs_oracle": err64_orc,
             "frame_err_vs_oracle": frame_err,
             "oracle_check": "source %d of %d, first %d of %d samples, %d frames, FP64 C port of the v6 loop; "
                             "max-normalised per model and DOF kind" % (r_mid, R, steps, n_t, fo.shape[1]),
             "frame_times_match": bool(np.array_equal(ft32, fto)),
             "_cpu_baseline": cpu}
    return fp64, gates


def subsection_rooflines(torch, bfe_gb300, models, offs, frc_dof, frc_rhs, frc_sig, mons, march32, R, n_t,
                         ti0, peak, dt, stream):
    """The coupled FMC model alone (its own plan) and the 32 sub-domain
    models alone (one multi-model plan), same march: DOF-updates/s and the
    step kernel's roofline."""
    main, subs = models[0], models[1:]
    steps_per_march = n_t - ti0
    out = {}

    def part_roofline(plan, dofs, rhs, fsig, mon, n_part, nnz_part, p_part):
        plan.set_timing(True)
        hist = torch.zeros((R, n_t, mon.size), dtype=torch.float64, device="cuda")
        march32(plan, hist, dofs, rhs, fsig, mon, R)
        torch.cuda.synchronize()
        st_ = plan.stats()
        plan.set_timing(False)
        ms_ = st_["step_ms"] / max(st_["step_launches"], 1)
        by = algorithmic_bytes(nnz_part, n_part, R, p_part, mon.size, 4)
        return {"n_dof": int(n_part), "step_kernel_ms": ms_, "achieved_gbs": by / ms_ / 1e6,
                "frac_of_measured_hbm": by / ms_ / 1e6 / peak,
                "kernel": KERNEL_NAMES.get(st_["variant"], "variant %d" % st_["variant"])}

    plan_a = bfe_gb300.Plan(main["K"], main["C"], main["M"], dt, bfe_gb300.VEL_CURRENT, "single", main["gl"])
    selm = frc_dof < offs[1]
    mons_a = mons[mons <= offs[1]]
    hist_a = torch.zeros((R, n_t, mons_a.size), dtype=torch.float64, device="cuda")
    march32(plan_a, hist_a, frc_dof[selm], frc_rhs[selm], frc_sig[selm], mons_a, R)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    march32(plan_a, hist_a, frc_dof[selm], frc_rhs[selm], frc_sig[selm], mons_a, R)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_a = e0.elapsed_time(e1)
    part_a = part_roofline(plan_a, frc_dof[selm], frc_rhs[selm], frc_sig[selm], mons_a, main["K"].shape[0],
                           main["K"].nnz, max(int((frc_rhs[selm] == r).sum()) for r in range(R)))
    plan_a.close()
    out["coupled_fmc_only"] = {"value": R * main["K"].shape[0] * steps_per_march / (ms_a * 1e-3), "unit": UNIT,
                               "ms_per_march": ms_a, "n_dof": int(main["K"].shape[0]), "roofline": part_a}
    if subs:
        plan_b, _ = bfe_gb300.Plan.multi([(m["K"], m["C"], m["M"], m["gl"]) for m in subs], dt,
                                         bfe_gb300.VEL_CURRENT, "single")
        sel_b = frc_dof >= offs[1]
        mons_b = mons[mons > offs[1]] - offs[1]
        out["subdomains_only"] = part_roofline(plan_b, frc_dof[sel_b] - offs[1], frc_rhs[sel_b], frc_sig[sel_b],
                                               mons_b, plan_b.n, sum(m["K"].nnz for m in subs),
                                               max(int((frc_rhs[sel_b] == r).sum()) for r in range(R)))
        plan_b.close()
    return out


def plate_c0_section(bfe_gb300, model):
    """The reference's CPU-runnable case: 20 x 10 mm steel plate at 0.1 mm
    (40,602 DOF, dof_to_use [1 2]), one top-centre point force, 16 top-surface
    monitors, 2,000 samples, a field frame every 500 samples, through the
    drop-in v6 call (plan creation, host buffers and copies included), FP64
    and FP32, against the FP64 C port of the v6 loop on all host threads.
    The model fits in L2."""
    from oracle import cpu_port
    m = model.steel_plate(W=20e-3, H=10e-3, h=0.1e-3, n_mon=16)
    n_t = 2000
    t = np.arange(n_t) * m["dt"]
    sig = model.toneburst(t, 5e6, 5)
    fi = model.global_indices(m["gl"], m["src_nodes"], 2)
    hi = model.global_indices(m["gl"], m["mon_nodes"], 2)
    res = {"n_dof": int(m["K"].shape[0]), "nnz_K": int(m["K"].nnz), "samples": n_t, "l2_resident": True}
    h64 = None
    for prec in ("double", "single"):
        best = 1e30
        for _ in range(3):
            t0 = time.perf_counter()
            h, fld, _, _ = bfe_gb300.fn_explicit_dynamic_solver_gb300(
                m["K"], m["C"], m["M"], t, fi, sig, [], [], hi, 500, 1, "KE", bfe_gb300.VEL_CURRENT, prec,
                gl_lookup=m["gl"])
            best = min(best, time.perf_counter() - t0)
        res[prec] = {"call_s": best, "dof_updates_per_s": m["K"].shape[0] * n_t / best}
        if prec == "double":
            h64 = h
        else:
            res[prec]["ascan_err_vs_fp64"] = float(np.abs(h - h64).max() / np.abs(h64).max())
    op = cpu_port.CpuOperator(m["K"], m["C"], m["M"], m["dt"])
    _, s = cpu_port.time_march(op, t, fi - 1, sig[None, :], hi - 1)
    res["cpu_port"] = {"s": s, "dof_updates_per_s": m["K"].shape[0] * n_t / s, "threads": cpu_port.threads()}
    res["speedup_fp64_call_vs_cpu"] = s / res["double"]["call_s"]
    return res


def coupled_c1_section(torch, bfe_gb300, model, main, peak, n_t=8000):
    """The coupled water/steel model on its own with one source (the array's
    centre element, pressure DOF), 8,000 samples, the 64 element centres
    monitored: one-source marches on resident FP64 and FP32 plans (host
    buffers), FP32 A-scans against FP64, and the step kernels' average launch
    (CUDA events) against the HBM roofline (R = 1 bytes)."""
    m = main
    n = int(m["K"].shape[0])
    t = np.arange(n_t) * m["dt"]
    sig = model.toneburst(t, 5e6, 5)
    fi = model.global_indices(m["gl"], m["src_nodes"][len(m["src_nodes"]) // 2], 4)
    hi = model.global_indices(m["gl"], m["mon_nodes"], 4)
    res = {"n_dof": n, "nnz_K": int(m["K"].nnz), "samples": n_t, "source_dofs": int(fi.size),
           "monitors": int(hi.size)}
    h64 = None
    for prec, b in (("double", 8), ("single", 4)):
        with bfe_gb300.Plan(m["K"], m["C"], m["M"], m["dt"], bfe_gb300.VEL_CURRENT, prec,
                            m["gl"] if prec == "single" else None, one_source=True) as plan:
            plan.run(t[:200], fi, sig[:200], hi)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            h, _, _ = plan.run(t, fi, sig, hi)
            el = time.perf_counter() - t0
            plan.set_timing(True)
            plan.run(t, fi, sig, hi)
            st = plan.stats()
            plan.set_timing(False)
        ms = st["step_ms"] / max(st["step_launches"], 1)
        by = algorithmic_bytes(m["K"].nnz, n, 1, fi.size, hi.size, b)
        res[prec] = {"march_s": el, "dof_updates_per_s": n * n_t / el, "step_kernel_ms": ms,
                     "achieved_gbs": by / ms / 1e6, "frac_of_measured_hbm": by / ms / 1e6 / peak,
                     "state_mb": 3 * n * b / 1e6}
        if prec == "double":
            h64 = h
        else:
            res[prec]["ascan_err_vs_fp64"] = float(np.abs(h - h64).max() / np.abs(h64).max())
    return res


def fmc_section(torch, bfe_gb300, d_hist, R, n_t, q, n_rx, sig, stream):
    """Full-matrix capture of the coupled model's array from the headline
    march's device history: 64 x 64 transmitter/receiver pairs gathered and
    convolved with the toneburst on the GPU (fn_parse_to_fmc), checked on 16
    pairs against the FFT convolution of fn_convolve on the host."""
    from bfe_gb300.fmc import fmc_from_device_history
    tx = [a for a in range(R) for _ in range(n_rx)]
    rx_slots = [[b] for _ in range(R) for b in range(n_rx)]
    rx_w = [[1.0]] * len(tx)
    d_out = torch.zeros((len(tx), n_t), dtype=torch.float64, device="cuda")
    fmc_from_device_history(d_hist, q, n_t, R, tx, rx_slots, rx_w, sig, d_out, stream.cuda_stream)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fmc_from_device_history(d_hist, q, n_t, R, tx, rx_slots, rx_w, sig, d_out, stream.cuda_stream)
    torch.cuda.synchronize()
    gpu_s = time.perf_counter() - t0
    out = d_out.cpu().numpy()
    hist = d_hist.cpu().numpy()
    rng = np.random.default_rng(5)
    picks = rng.choice(len(tx), 16, replace=False)
    t0 = time.perf_counter()
    errs = []
    for k in picks:
        trace = hist[tx[k], :, rx_slots[k][0]]
        F = np.fft.fft(trace, 2 * n_t) * np.fft.fft(sig, 2 * n_t)
        ref = np.fft.ifft(F).real[:n_t]
        errs.append(float(np.abs(out[k] - ref).max() / max(np.abs(ref).max(), 1e-300)))
    host_per_pair = (time.perf_counter() - t0) / len(picks)
    return {"pairs": len(tx), "samples": n_t, "gpu_s": gpu_s, "host_fft_s_per_pair": host_per_pair,
            "host_fft_s_all_pairs_estimate": host_per_pair * len(tx), "max_rel_err_vs_fft_16_pairs": max(errs)}


def assembly_section(torch, bfe_gb300, model, m):
    """Global assembly of the coupled 60 x 30 mm model (1.44M triangles plus
    the ASI2D2 interface) on the GPU (bfe_assemble_2d) against the vectorised
    host builder, and the plan built from the device matrices."""
    args = (m["nds"], m["els"], m["el_mat"], m["el_abs"], m["typ"], m["matls"])
    kw = dict(dof_to_use=(1, 2, 4), damping_power_law=2)
    t0 = time.perf_counter()
    Kh, Ch, Mh, glh = model.assemble(*args, **kw)
    host_s = time.perf_counter() - t0
    with bfe_gb300.DeviceMatrices(*args, **kw):          # first call: module load
        pass
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dm = bfe_gb300.DeviceMatrices(*args, **kw)
    gpu_s = time.perf_counter() - t0
    with dm:
        t0 = time.perf_counter()
        with dm.plan(m["dt"], bfe_gb300.VEL_CURRENT, "single"):
            plan_s = time.perf_counter() - t0
        err = max(float(abs(dm.matrix(k) - X).max() / abs(X).max()) for k, X in enumerate((Kh, Ch, Mh)))
        same_gl = bool(np.array_equal(dm.gl_lookup(), glh))
    return {"elements": int(len(m["els"])), "n_dof": int(Kh.shape[0]), "nnz_K": int(Kh.nnz),
            "host_assembly_s": host_s, "gpu_assembly_s": gpu_s, "speedup": host_s / gpu_s,
            "plan_from_device_matrices_s": plan_s, "max_rel_diff_vs_host": err, "same_gl_lookup": same_gl,
            "note": "GPU time includes mesh upload and the sort; plan creation is host code"}


def hex3d_section(torch, bfe_gb300, model):
    """3D steel block of 8-node bricks (10 x 10 x 5 mm at 0.1 mm, 500,000
    bricks): one source, 3,000 samples, FP32 and FP64 marches, roofline of
    the step kernel and the FP32 A-scan error against FP64."""
    m = model.steel_block_3d()
    n_t = 3000
    dt = m["dt"]
    t = np.arange(n_t) * dt
    sig = model.toneburst(t, 5e6, 5)
    fi = model.global_indices(m["gl"], m["src_nodes"][0], 3)
    hi = model.global_indices(m["gl"], m["mon_nodes"], 3)
    n = m["K"].shape[0]
    nnz = m["K"].nnz
    out = {"n_dof": n, "nnz_K": int(nnz), "samples": n_t, "monitors": int(hi.size)}
    hists = {}
    peak, _ = measured_peak_hbm()
    for prec, b in (("single", 4), ("double", 8)):
        with bfe_gb300.Plan(m["K"], m["C"], m["M"], dt, bfe_gb300.VEL_CURRENT, prec, m["gl"]) as p:
            p.run(t[:100], fi, sig[:100], hi)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            h, _, _ = p.run(t, fi, sig, hi)
            el = time.perf_counter() - t0
            hists[prec] = h
            p.set_timing(True)
            p.run(t[:300], fi, sig[:300], hi)
            st = p.stats()
        step_ms = st["step_ms"] / max(st["step_launches"], 1)
        gbs = algorithmic_bytes(nnz, n, 1, 1, hi.size, b) / (step_ms * 1e-3) / 1e9
        out["fp32" if b == 4 else "fp64"] = {"value": n * n_t / el, "unit": UNIT, "march_s": el,
                                            "step_kernel_ms": step_ms, "achieved_gbs": gbs,
                                            "frac_of_measured_hbm": gbs / peak}
    out["ascan_err_fp32_vs_fp64"] = float(np.abs(hists["single"] - hists["double"]).max() /
                                          np.abs(hists["double"]).max())
    return out


def adjoint_section(torch, bfe_gb300, model, n_fd=20, n_t=4000):
    """Adjoint gradient on the 30 x 15 mm steel plate at 0.05 mm (~360k
    triangles): 16 sources x 16 receivers, 4,000 samples, observed A-scans
    from a seeded +-5 % stiffness perturbation (1 mm Gaussian bumps),
    gradient of the misfit w.r.t. per-element stiffness scale and density
    (backward segments of sqrt(N) steps; forward states kept on the device
    when they fit) in FP32 and FP64, FP64 central differences on n_fd random
    elements of the sensitive region."""
    m = model.steel_plate_adjoint()
    ke, mh, ch, dof = m["element_data"]
    n = m["K"].shape[0]
    dt = m["dt"]
    t = np.arange(n_t) * dt
    sig = model.toneburst(t, 5e6, 5)
    srcs = [model.global_indices(m["gl"], s_, 2) for s_ in m["src_nodes"]]
    rec = model.global_indices(m["gl"], m["rec_nodes"], 2)
    rho_e = np.full(len(dof), m["rho"])
    Kt, Ct, Mt = model.assemble_from_elements(ke, mh, ch, dof, n, m["s_true"], rho_e)
    with bfe_gb300.Plan(Kt, Ct, Mt, dt, bfe_gb300.VEL_CURRENT, "double") as p:
        obs = p.run_batched(t, srcs, sig, rec)
    K0, C0, M0 = model.assemble_from_elements(ke, mh, ch, dof, n, None, rho_e)
    res = {"n_dof": n, "elements": int(len(dof)), "sources": len(srcs), "receivers": int(rec.size),
           "samples": n_t, "segment_steps": int(np.ceil(np.sqrt(n_t)))}
    grads = {}
    for prec in ("single", "double"):
        with bfe_gb300.Plan(K0, C0, M0, dt, bfe_gb300.VEL_CURRENT, prec, m["gl"]) as p:
            p.adjoint_gradient((ke, mh, ch, dof), t[:200], srcs, sig, rec, obs[:, :200, :])
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            J, gs, gr = p.adjoint_gradient((ke, mh, ch, dof), t, srcs, sig, rec, obs)
            el = time.perf_counter() - t0
            kept = p.stats()["adjoint_kept"]
        grads[prec] = (J, gs, gr)
        res["fp32" if prec == "single" else "fp64"] = {
            "gradient_s": el, "misfit": J,
            "forward_states": "kept on the device" if kept else "recomputed from checkpoints"}
    J64, gs64, gr64 = grads["double"]
    _, gs32, gr32 = grads["single"]
    res["fp32_vs_fp64_rel"] = {"stiffness": float(np.linalg.norm(gs32 - gs64) / np.linalg.norm(gs64)),
                               "density": float(np.linalg.norm(gr32 - gr64) / np.linalg.norm(gr64))}
    if n_fd < 1:
        return res
    rng = np.random.default_rng(3)
    sens = np.nonzero(np.abs(gs64) >= 1e-2 * np.abs(gs64).max())[0]
    picks = rng.choice(sens, min(n_fd, sens.size), replace=False)

    import scipy.sparse as sp

    def element_block(e, vals):
        """Sparse n x n matrix holding one element's ndf x ndf block."""
        d = dof[e]
        ok = d >= 0
        d = d[ok]
        v = np.asarray(vals)[np.ix_(ok, ok)] if np.ndim(vals) == 2 else np.diag(np.asarray(vals)[ok])
        return sp.csr_matrix((v.T.ravel(), (np.repeat(d, d.size), np.tile(d, d.size))), shape=(n, n))

    def J_at(dK=None, dM=None, dC=None):
        K = K0 if dK is None else (K0 + dK).tocsr()
        M = M0 if dM is None else (M0 + dM).tocsr()
        C = C0 if dC is None else (C0 + dC).tocsr()
        with bfe_gb300.Plan(K, C, M, dt, bfe_gb300.VEL_CURRENT, "double") as p:
            h = p.run_batched(t, srcs, sig, rec)
        return 0.5 * ((h - obs) ** 2).sum()
    t0 = time.perf_counter()
    errs_s, errs_r = [], []
    for e in picks:
        eps = 1e-3
        dk = element_block(e, ke[e]) * eps                  # s_e = 1 +- eps
        fd = (J_at(dK=dk) - J_at(dK=-dk)) / (2 * eps)
        errs_s.append(abs(gs64[e] - fd) / abs(fd))
        dm = element_block(e, mh[e]) * (eps * rho_e[e])     # rho_e (1 +- eps)
        dc = element_block(e, ch[e]) * (eps * rho_e[e])
        fdr = (J_at(dM=dm, dC=dc) - J_at(dM=-dm, dC=-dc)) / (2 * eps * rho_e[e])
        errs_r.append(abs(gr64[e] - fdr) / abs(fdr))
    res["finite_difference"] = {"elements": int(len(picks)), "max_rel_err_stiffness": float(max(errs_s)),
                                "max_rel_err_density": float(max(errs_r)), "seconds": time.perf_counter() - t0,
                                "selection": "random elements with |dJ/ds| >= 1e-2 max"}
    return res


def cpu_baseline(K, C, M, dt, t, src_gi, sig, mons, target_s=10.0, n_frames=4):
    """The FP64 CPU restatement of the reference's time loop (oracle port) on
    all host threads, timed on a bounded prefix of one source's march. The
    timed march also writes n_frames field frames (velocity); returns the
    baseline dict and (history q x steps, frames, frame times, steps,
    frame interval) for the oracle checks."""
    from oracle import cpu_port
    op = cpu_port.CpuOperator(K, C, M, dt)
    n = K.shape[0]
    probe = 20
    _, s = cpu_port.time_march(op, t[:probe], src_gi - 1, sig[None, :probe], mons - 1)
    steps = int(min(len(t), max(probe, target_s / max(s / probe, 1e-9))))
    every = max(1, -(-steps // n_frames))
    t0 = time.perf_counter()
    hist, fld, fld_t = op.march(t[:steps], src_gi - 1, sig[None, :steps], mons - 1, every, True, frames=True)
    s = time.perf_counter() - t0
    return ({"value": n * steps / s, "unit": UNIT, "cores": cpu_port.threads(), "kind": "port",
             "sample": "one source, first %d of %d samples, %d velocity frames, FP64 v6 loop (C, OpenMP)"
                       % (steps, len(t), fld.shape[1])},
            (hist, fld, fld_t, steps, every))


def _ref_subdomain(args):
    """Worker: one steel sub-domain model (square with absorbing layers on
    every side and a seeded void blob) built with the oracle's restatements
    of the reference's mesh and assembly code; returns (K, C, M, dt). The
    geometry is our arm's (same void polygon for the seed, absorbers
    min(3 wavelengths, side / 4) thick, quadratic grading), so both arms march
    the same matrices."""
    from oracle import assembly, mesh, signals
    side, seed, h, fc = args
    steel = dict(rho=8000.0, D=signals.isotropic_stiffness_matrix(210e9, 0.3), el_typ="CPE3")
    mod = mesh.rectangular_structured_mesh(np.array([[0, 0], [side, 0], [side, side], [0, side]]), h)
    blob = blob_polygon(min(1.5e-3, side / 8), (side / 2, side / 2), seed)
    mod = mesh.remove_elements_in_region(mod, blob)
    cL = np.sqrt(steel["D"][0, 0] / steel["rho"])
    th = min(3.0 * cL / fc, side / 4)
    inner = np.array([[th, th], [side - th, th], [side - th, side - th], [th, side - th]])
    mod = mesh.add_absorbing_layer(mod, inner, th)
    mod["el_typ_i"] = ["CPE3"] * len(mod["el_mat_i"])
    K, C, M, _ = assembly.build_global_matrices_v5(mod["nds"], mod["els"], mod["el_mat_i"], mod["el_abs_i"],
                                                   mod["el_typ_i"], [steel],
                                                   dict(dof_to_use=[1, 2], damping_power_law=2))
    dt = signals.element_eigen_time_step(mod["nds"], mod["els"], steel["D"], steel["rho"])
    return K, C, M, dt


def run_reference(args):
    """The reference's CPU path (FP64 oracle port of the v6 loop on all host
    threads) on the same workload - the coupled model and the sub-domain
    models joined into one operator, built with the oracle's restatements of
    the reference's mesh and assembly code - each step a bounded sample of
    one source's march."""
    rank = int(os.environ.get("RANK", 0))
    if rank != 0:
        return None
    import shutil
    # the reference itself is MATLAB code: record whether a MATLAB or GNU
    # Octave runtime exists on this machine (the timed path is the oracle's C
    # port of its v6 loop when neither does)
    runtime_probe = {k: shutil.which(k) for k in ("matlab", "octave", "octave-cli")}
    from oracle import assembly, cpu_port, mesh, signals
    w = workload(args.scale)
    if args.sources:
        w["n_src"] = args.sources
    n_t = args.n_t or w["n_t"]
    steel = dict(rho=8000.0, D=signals.isotropic_stiffness_matrix(210e9, 0.3), el_typ="CPE3")
    water = dict(rho=1000.0, D=1500.0 ** 2 * 1000.0, el_typ="AC2D3")
    matls = [steel, water]
    Ht = w["H_water"] + w["H_steel"]
    mod = mesh.rectangular_structured_mesh(np.array([[0, 0], [w["W"], 0], [w["W"], Ht], [0, Ht]]), w["h"])
    mod = mesh.set_els_inside_bdry_to_mat(
        mod, np.array([[-1, w["H_steel"]], [w["W"] + 1, w["H_steel"]], [w["W"] + 1, Ht + 1], [-1, Ht + 1]]), 2)
    mod = mesh.remove_elements_in_region(mod, w["blob"])
    mod["el_typ_i"] = [matls[k - 1]["el_typ"] for k in mod["el_mat_i"]]
    cL = np.sqrt(steel["D"][0, 0] / steel["rho"])
    th = 3.0 * cL / w["fc"]
    inner = np.array([[th, th], [w["W"] - th, th], [w["W"] - th, Ht + 1.0], [th, Ht + 1.0]])
    mod = mesh.add_absorbing_layer(mod, inner, th)
    mod = mesh.add_fluid_solid_interface_els(mod, matls)
    K, C, M, gl = assembly.build_global_matrices_v5(mod["nds"], mod["els"], mod["el_mat_i"], mod["el_abs_i"],
                                                    mod["el_typ_i"], matls,
                                                    dict(dof_to_use=[1, 2, 4], damping_power_law=2))
    solid = np.array([x == "CPE3" for x in mod["el_typ_i"]])
    dt = signals.element_eigen_time_step(mod["nds"], mod["els"][solid, :3], steel["D"], steel["rho"])
    t = np.arange(n_t) * dt
    sig = signals.gaussian_pulse(t, w["fc"], w["cycles"])
    top = np.nonzero(np.isclose(mod["nds"][:, 1], Ht))[0]
    xc = w["W"] / 2 + (np.arange(w["n_src"]) - (w["n_src"] - 1) / 2) * w["pitch"]
    mid = top[np.abs(mod["nds"][top, 0] - xc[w["n_src"] // 2]) <= 0.4 * w["pitch"] + 1e-12] + 1
    src = gl[mid - 1, 3]
    src = src[src > 0]
    mons = np.array([gl[top[np.argmin(np.abs(mod["nds"][top, 0] - x))], 3] for x in xc])
    n_models = 1
    if args.subdomains:
        import multiprocessing as mp
        import scipy.sparse as sp
        from concurrent.futures import ProcessPoolExecutor
        from bfe_gb300.model import subdomain_sides
        sides = subdomain_sides(args.subdomains, h=w["h"]) * args.scale
        with ProcessPoolExecutor(max_workers=min(args.subdomains, os.cpu_count() or 4),
                                 mp_context=mp.get_context("spawn")) as ex:
            subs = list(ex.map(_ref_subdomain, [(float(sd), 100 + k, w["h"], w["fc"])
                                                for k, sd in enumerate(sides)]))
        K = sp.block_diag([K] + [x[0] for x in subs], format="csr")
        C = sp.block_diag([C] + [x[1] for x in subs], format="csr")
        M = sp.block_diag([M] + [x[2] for x in subs], format="csr")
        dt = min([dt] + [x[3] for x in subs])
        t = np.arange(n_t) * dt
        sig = signals.gaussian_pulse(t, w["fc"], w["cycles"])
        n_models += len(subs)
    op = cpu_port.CpuOperator(K, C, M, dt)
    n = K.shape[0]
    probe = 10
    _, s = cpu_port.time_march(op, t[:probe], src - 1, sig[None, :probe], mons - 1)
    per = max(s / probe, 1e-9)
    steps = int(min(n_t, max(probe, 8.0 / per)))
    for _ in range(args.warmup):
        cpu_port.time_march(op, t[:steps], src - 1, sig[None, :steps], mons - 1)
    secs = []
    for _ in range(args.steps):
        _, s = cpu_port.time_march(op, t[:steps], src - 1, sig[None, :steps], mons - 1)
        secs.append(s)
    s = sum(secs) / len(secs)
    value = n * steps / s
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": int(os.environ.get("WORLD_SIZE", 1)), "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": s * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": workload_config(w, n_models - 1, n_t, n_t - int(np.nonzero(sig)[0].min()), n,
                                  K.count_nonzero(), n_models, w["n_src"] + (n_models - 1) * SUB_MONITORS,
                                  int(os.environ.get("WORLD_SIZE", 1)), args.scale),
        "run": {"kernel_path": "reference CPU v6 loop (FP64, the oracle's C port), the models joined in one "
                               "operator, one source per bounded sample",
                "sample_steps": steps},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cpu_port.threads(), "kind": "port",
                         "sample": "first %d of %d samples of one source" % (steps, n_t)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_runtime_probe": runtime_probe,
    }
    print(json.dumps(line), flush=True)
    return line


def run_only(args):
    """One extra section alone on cuda:0 (profiling runs)."""
    import torch
    import bfe_gb300
    from bfe_gb300 import model
    torch.cuda.set_device(0)
    bfe_gb300.load()
    if args.only == "c1":
        w = workload(1.0)
        main = model.coupled_water_steel(W=w["W"], H_water=w["H_water"], H_steel=w["H_steel"], h=w["h"],
                                         fc=w["fc"], blob_polygon_pts=w["blob"], array_elements=w["n_src"],
                                         array_pitch=w["pitch"])
        res = coupled_c1_section(torch, bfe_gb300, model, main, measured_peak_hbm()[0], n_t=args.n_t or 8000)
        print(json.dumps({"section": "coupled_c1", **res}), flush=True)
        return
    res = adjoint_section(torch, bfe_gb300, model, n_fd=0, n_t=args.n_t or 4000)
    print(json.dumps({"section": "adjoint_c4", **res}), flush=True)


def main():
    args = parse()
    if args.only:
        run_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
