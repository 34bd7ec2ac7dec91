"""GPU parity: the native kernels (through the C ABI) against the FP64 oracle.

Tolerances: max-normalised error max|gpu - oracle| / max|oracle| of each
result, <= 1e-10 for FP64 plans and <= 1e-4 for FP32 plans (the acceptance
bound for FP32 A-scans)."""
import numpy as np
import pytest

import modelgen
from oracle import solver as osolver

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
TOL32 = 1e-4


def _err(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def bfe():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from bfe_gb300 import _lib, build
    build.build()
    import bfe_gb300
    bfe_gb300.load()
    return bfe_gb300


def _oracle(m, t, fi, F, hi, every=np.inf, ftype="KE", mode=osolver.VEL_CURRENT):
    return osolver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, fi, F, [], [], hi,
                                              every, 0, ftype, mode)


@pytest.fixture(scope="module")
def plate():
    return modelgen.solid_plate(W=4e-3, H=2e-3, h=0.1e-3, dof_to_use=(1, 2))


@pytest.fixture(scope="module")
def coupled():
    return modelgen.coupled_model(W=3e-3, Hw=1.5e-3, Hs=1.5e-3, h=0.1e-3, abs_thick=0.6e-3, blob=True)


@pytest.mark.parametrize("prec,tol", [("double", TOL64), ("single", TOL32)])
def test_solid_plate_history_and_frames(bfe, plate, prec, tol):
    m = plate
    nt = 700
    t, s = modelgen.pulse(nt, m["dt"])
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    hi = modelgen.gi_of(m["gl"], m["mon_nds"], 2)
    h0, f0, _, ft0 = _oracle(m, t, fi, s, hi, every=175)
    h1, f1, frc, ft1 = bfe.fn_explicit_dynamic_solver_gb300(
        m["K"], m["C"], m["M"], t, fi, s, [], [], hi, 175, 1, "KE", osolver.VEL_CURRENT, prec,
        gl_lookup=m["gl"])
    assert frc is None
    assert h1.shape == h0.shape and f1.shape == f0.shape
    assert _err(h1, h0) <= tol
    assert _err(f1, f0) <= tol
    assert np.array_equal(ft1, ft0)


@pytest.mark.parametrize("mode", [osolver.VEL_CURRENT, osolver.VEL_LAST_HALF])
@pytest.mark.parametrize("prec,tol", [("double", TOL64), ("single", TOL32)])
def test_coupled_fluid_solid_with_absorbers(bfe, coupled, mode, prec, tol):
    m = coupled
    nt = 500
    t, s = modelgen.pulse(nt, m["dt"])
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 4)          # pressure source in the water
    hi = np.concatenate([modelgen.gi_of(m["gl"], m["mon_nds"], 4),
                         modelgen.gi_of(m["gl"], m["mon_nds"], 2)])
    h0, _, _, _ = _oracle(m, t, fi, s, hi, mode=mode)
    h1, _, _, _ = bfe.fn_explicit_dynamic_solver_gb300(
        m["K"], m["C"], m["M"], t, fi, s, [], [], hi, np.inf, 1, "KE", mode, prec, gl_lookup=m["gl"])
    assert np.isfinite(h0).all()
    # fluid (pressure) and solid (displacement) rows have different units:
    # normalise each family separately
    q4 = modelgen.gi_of(m["gl"], m["mon_nds"], 4).size
    assert _err(h1[:q4], h0[:q4]) <= tol
    assert _err(h1[q4:], h0[q4:]) <= tol


@pytest.mark.parametrize("prec,tol", [("double", TOL64), ("single", TOL32)])
def test_forcing_rows_duplicates_and_start(bfe, plate, prec, tol):
    m = plate
    nt = 300
    t, s = modelgen.pulse(nt, m["dt"])
    s = np.concatenate([np.zeros(37), s[:-37]])             # ti_start = 38 (1-based)
    nds = [m["frc_nd"], m["frc_nd"] - 1, m["frc_nd"] + 1, m["frc_nd"]]
    fi = modelgen.gi_of(m["gl"], nds, 2)                     # duplicate DOF: last row wins
    F = np.vstack([s, 0.5 * s, -0.25 * s, 2.0 * s])
    hi = np.concatenate([fi, modelgen.gi_of(m["gl"], m["mon_nds"], 1)])
    h0, _, _, _ = _oracle(m, t, fi, F, hi)
    h1, _, _, _ = bfe.fn_explicit_dynamic_solver_gb300(
        m["K"], m["C"], m["M"], t, fi, F, [], [], hi, np.inf, 1, "KE", osolver.VEL_CURRENT, prec,
        gl_lookup=m["gl"])
    assert np.all(h1[:, :37] == 0)
    assert _err(h1, h0) <= tol


def test_zero_forcing_runs_no_steps(bfe, plate):
    m = plate
    t = np.arange(50) * m["dt"]
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    h1, f1, _, ft = bfe.fn_explicit_dynamic_solver_gb300(
        m["K"], m["C"], m["M"], t, fi, np.zeros(50), [], [], fi, 10, 1, "KE", osolver.VEL_CURRENT, "double")
    assert np.all(h1 == 0) and np.all(f1 == 0) and np.all(ft == 0)


def test_displacement_field_output(bfe, plate):
    m = plate
    nt = 200
    t, s = modelgen.pulse(nt, m["dt"])
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    h0, f0, _, ft0 = _oracle(m, t, fi, s, fi, every=33, ftype="mean(u2)")
    h1, f1, _, ft1 = bfe.fn_explicit_dynamic_solver_gb300(
        m["K"], m["C"], m["M"], t, fi, s, [], [], fi, 33, 1, "mean(u2)", osolver.VEL_CURRENT, "double")
    assert _err(f1, f0) <= TOL64 and np.array_equal(ft0, ft1)


@pytest.mark.parametrize("prec", ["double", "single"])
def test_batched_sources_equal_single_runs(bfe, coupled, prec):
    m = coupled
    nt = 300
    t, s = modelgen.pulse(nt, m["dt"])
    top = m["mon_nds"][:4]
    srcs = [modelgen.gi_of(m["gl"], [nd], 4) for nd in top]
    hi = np.concatenate([modelgen.gi_of(m["gl"], m["mon_nds"], 4),
                         modelgen.gi_of(m["gl"], m["mon_nds"], 2)])
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], osolver.VEL_CURRENT, prec, m["gl"]) as plan:
        hb = plan.run_batched(t, srcs, s, hi)
        # the one-source path sums the interface correction in another order,
        # so the paths agree to the rounding of the precision
        same = 1e-12 if prec == "double" else 1e-6
        for r, fi in enumerate(srcs):
            h1, _, _ = plan.run(t, fi, s, hi)
            assert np.abs(hb[:, :, r] - h1).max() <= same * max(np.abs(h1).max(), 1e-300)
    # and against the oracle for one source
    h0, _, _, _ = _oracle(m, t, srcs[1], s, hi)
    q4 = modelgen.gi_of(m["gl"], m["mon_nds"], 4).size
    tol = TOL64 if prec == "double" else TOL32
    assert _err(hb[:q4, :, 1], h0[:q4]) <= tol


def test_batched_64_sources_fp32(bfe, coupled):
    m = coupled
    nt = 200
    t, s = modelgen.pulse(nt, m["dt"])
    nds = np.nonzero(m["gl"][:, 3] > 0)[0] + 1
    srcs = [modelgen.gi_of(m["gl"], [nds[(7 * r) % nds.size]], 4) for r in range(64)]
    hi = modelgen.gi_of(m["gl"], m["mon_nds"], 4)
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], osolver.VEL_CURRENT, "single", m["gl"]) as plan:
        hb = plan.run_batched(t, srcs, s, hi)
    for r in (0, 17, 63):
        h0, _, _, _ = _oracle(m, t, srcs[r], s, hi)
        assert _err(hb[:, :, r], h0) <= TOL32


def test_errors_through_the_abi(bfe, plate):
    m = plate
    t = np.arange(20) * m["dt"]
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"]) as plan:
        with pytest.raises(bfe.BfeError) as ei:
            plan.run(t, [m["K"].shape[0] + 5], np.ones(20), [1])
        assert ei.value.status == 1
        with pytest.raises(bfe.BfeError):
            plan.run(t * 2, [1], np.ones(20), [1])                 # dt mismatch
        with pytest.raises(bfe.BfeError):
            plan.run(t, [1, 2], np.ones((3, 20)), [1])             # 3 rows for 2 DOFs


@pytest.mark.parametrize("variant", [0, 9, 10, 11, 12, 13, 14, 20, 22])
def test_every_batched_fp32_kernel_variant(bfe, coupled, variant, monkeypatch):
    """Each batched FP32 kernel (forced through BFE_VARIANT) gives the same
    answers: 0 the slice-staged row kernel, 9-14 the packed warp-per-node
    group kernel, 20 and 22 the half-warp float4 group kernel."""
    m = coupled
    nt = 150
    t, s = modelgen.pulse(nt, m["dt"])
    nds = np.nonzero(m["gl"][:, 3] > 0)[0] + 1
    srcs = [modelgen.gi_of(m["gl"], [nds[(11 * r) % nds.size]], 4) for r in range(64)]
    hi = np.concatenate([modelgen.gi_of(m["gl"], m["mon_nds"], 4),
                         modelgen.gi_of(m["gl"], m["mon_nds"], 2)])
    q4 = modelgen.gi_of(m["gl"], m["mon_nds"], 4).size
    monkeypatch.setenv("BFE_VARIANT", str(variant))
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], osolver.VEL_CURRENT, "single", m["gl"]) as plan:
        hb = plan.run_batched(t, srcs, s, hi)
        st = plan.stats()
    assert st["variant"] == variant
    assert st["n_nodes"] > 0 and st["n_groups"] == 2          # solid {1,2}, fluid {4}
    for r in (0, 33):
        h0, _, _, _ = _oracle(m, t, srcs[r], s, hi)
        assert _err(hb[:q4, :, r], h0[:q4]) <= TOL32
        assert _err(hb[q4:, :, r], h0[q4:]) <= TOL32


@pytest.mark.parametrize("R", [16, 32])
@pytest.mark.parametrize("variant", [0, 20, 22])
def test_half_warp_kernels_with_16_and_32_sources(bfe, coupled, R, variant, monkeypatch):
    """The half-warp group kernels with 4 (R = 16) or 8 (R = 32) lanes per
    node, and the slice kernel, against the oracle."""
    m = coupled
    nt = 150
    t, s = modelgen.pulse(nt, m["dt"])
    nds = np.nonzero(m["gl"][:, 3] > 0)[0] + 1
    srcs = [modelgen.gi_of(m["gl"], [nds[(13 * r) % nds.size]], 4) for r in range(R)]
    hi = np.concatenate([modelgen.gi_of(m["gl"], m["mon_nds"], 4), modelgen.gi_of(m["gl"], m["mon_nds"], 2)])
    monkeypatch.setenv("BFE_VARIANT", str(variant))
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], osolver.VEL_CURRENT, "single", m["gl"]) as plan:
        hb = plan.run_batched(t, srcs, s, hi)
        assert plan.stats()["variant"] == variant
    for r in (0, R - 1):
        h0, _, _, _ = _oracle(m, t, srcs[r], s, hi)
        assert _err(hb[:, :, r], h0) <= TOL32


@pytest.mark.parametrize("R,variant", [(64, 0), (64, 1), (64, 2), (64, 3), (32, 2), (32, 3), (16, 3)])
def test_fp64_group_kernels(bfe, coupled, R, variant, monkeypatch):
    """FP64 plans with node information march many sources with the FP64
    group block-sparse kernel (direct form); variant 0 is the slice kernel."""
    m = coupled
    nt = 150
    t, s = modelgen.pulse(nt, m["dt"])
    nds = np.nonzero(m["gl"][:, 3] > 0)[0] + 1
    srcs = [modelgen.gi_of(m["gl"], [nds[(7 * r) % nds.size]], 4) for r in range(R)]
    hi = np.concatenate([modelgen.gi_of(m["gl"], m["mon_nds"], 4), modelgen.gi_of(m["gl"], m["mon_nds"], 2)])
    monkeypatch.setenv("BFE_VARIANT", str(variant))
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], osolver.VEL_CURRENT, "double", m["gl"]) as plan:
        hb = plan.run_batched(t, srcs, s, hi)
        assert plan.stats()["variant"] == variant
    for r in (0, R - 1):
        h0, _, _, _ = _oracle(m, t, srcs[r], s, hi)
        assert _err(hb[:, :, r], h0) <= TOL64


@pytest.mark.parametrize("prec,tol", [("double", TOL64), ("single", TOL32)])
def test_multi_model_plan_matches_each_model(bfe, plate, coupled, prec, tol):
    """Independent models joined block-diagonally in one plan: each model's
    A-scans equal its own oracle run."""
    nt = 240
    t, s = modelgen.pulse(nt, min(plate["dt"], coupled["dt"]))
    dt = t[1] - t[0]
    plan, offs = bfe.Plan.multi([(plate["K"], plate["C"], plate["M"], plate["gl"]),
                                 (coupled["K"], coupled["C"], coupled["M"], coupled["gl"])],
                                dt, osolver.VEL_CURRENT, prec)
    with plan:
        f0 = modelgen.gi_of(plate["gl"], [plate["frc_nd"]], 2)
        f1 = modelgen.gi_of(coupled["gl"], [coupled["frc_nd"]], 4)
        h0i = modelgen.gi_of(plate["gl"], plate["mon_nds"], 2)
        h1i = modelgen.gi_of(coupled["gl"], coupled["mon_nds"], 4)
        hist = plan.run_batched(t, [f0, f1 + offs[1]], s, np.concatenate([h0i, h1i + offs[1]]))
    for k, (m, fi, hi) in enumerate(((plate, f0, h0i), (coupled, f1, h1i))):
        mm = dict(m)
        ref, _, _, _ = osolver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, fi, s, [], [], hi,
                                                          np.inf, 0, "KE", osolver.VEL_CURRENT)
        got = hist[:h0i.size, :, 0] if k == 0 else hist[h0i.size:, :, 1]
        assert _err(got, ref) <= tol
    # the other model's source does not leak across the block diagonal
    assert np.all(hist[:h0i.size, :, 1] == 0) and np.all(hist[h0i.size:, :, 0] == 0)


@pytest.mark.parametrize("prec", ["double", "single"])
def test_graph_replay_equals_plain_launches(bfe, coupled, prec, monkeypatch):
    m = coupled
    nt = 400                                   # >= 2 graph chunks of 48 steps plus a tail
    t, s = modelgen.pulse(nt, m["dt"])
    srcs = [modelgen.gi_of(m["gl"], [nd], 4) for nd in m["mon_nds"][:3]]
    hi = modelgen.gi_of(m["gl"], m["mon_nds"], 4)
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], osolver.VEL_CURRENT, prec, m["gl"]) as plan:
        hg = plan.run_batched(t, srcs, s, hi)
        monkeypatch.setenv("BFE_NO_GRAPH", "1")
        hp = plan.run_batched(t, srcs, s, hi)
    assert np.array_equal(hg, hp)


@pytest.mark.parametrize("prec,tol", [("double", TOL64), ("single", TOL32)])
def test_128_sources_take_two_chunks_per_lane(bfe, coupled, prec, tol):
    """R = 128: the batched kernels loop over two 64-source chunks per lane
    (FP32 half-warp kernels, FP64 group kernels); sources from both chunks
    match the oracle."""
    m = coupled
    nt = 150
    t, s = modelgen.pulse(nt, m["dt"])
    nds = np.nonzero(m["gl"][:, 3] > 0)[0] + 1
    R = 128
    srcs = [modelgen.gi_of(m["gl"], [nds[(5 * r) % nds.size]], 4) for r in range(R)]
    hi = np.concatenate([modelgen.gi_of(m["gl"], m["mon_nds"], 4), modelgen.gi_of(m["gl"], m["mon_nds"], 2)])
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], osolver.VEL_CURRENT, prec, m["gl"]) as plan:
        hb = plan.run_batched(t, srcs, s, hi)
        st = plan.stats()
    assert st["n_groups"] == 2
    for r in (0, 63, 64, 127):
        h0, _, _, _ = _oracle(m, t, srcs[r], s, hi)
        assert _err(hb[:, :, r], h0) <= tol, r


def test_autotuner_choice_is_kept_across_plans(bfe, monkeypatch):
    """The first batched run of an operator shape times the candidate
    kernels; a second plan over the same operator reuses the choice without
    timing them again (fewer auxiliary launches), and its results match."""
    monkeypatch.delenv("BFE_VARIANT", raising=False)
    # a model size no other test uses, so that no earlier run has tuned it
    m = modelgen.coupled_model(W=2.3e-3, Hw=1.1e-3, Hs=1.2e-3, h=0.1e-3, abs_thick=0.4e-3)
    nt = 120
    t, s = modelgen.pulse(nt, m["dt"])
    nds = np.nonzero(m["gl"][:, 3] > 0)[0] + 1
    srcs = [modelgen.gi_of(m["gl"], [nds[(5 * r) % nds.size]], 4) for r in range(64)]
    hi = modelgen.gi_of(m["gl"], m["mon_nds"], 4)
    runs = []
    for _ in range(2):
        with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], osolver.VEL_CURRENT, "single", m["gl"]) as plan:
            h = plan.run_batched(t, srcs, s, hi)
            runs.append((h, plan.stats()))
    (h1, s1), (h2, s2) = runs
    assert s1["variant"] == s2["variant"] in (20, 22)
    assert s2["aux_launches"] < s1["aux_launches"]
    assert np.array_equal(h1, h2)
