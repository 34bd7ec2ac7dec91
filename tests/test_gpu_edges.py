"""Edge cases through the C ABI against the FP64 oracle: no forcing, no
monitors, the shortest time axis, frames sparser than the run, ragged
source sets (with and without the 64-RHS kernels), a forced and monitored
DOF, per-source signals, repeated monitors. Tolerances as the parity tests:
1e-10 (FP64), 1e-4 (FP32), max-normalised."""
import numpy as np
import pytest

import modelgen
from oracle import solver as osolver

pytestmark = pytest.mark.gpu

TOL = {"double": 1e-10, "single": 1e-4}


def _err(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def bfe():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from bfe_gb300 import build
    build.build()
    import bfe_gb300
    bfe_gb300.load()
    return bfe_gb300


@pytest.fixture(scope="module")
def plate():
    return modelgen.solid_plate(W=3e-3, H=1.5e-3, h=0.1e-3, dof_to_use=(1, 2), abs_thick=0.4e-3)


def _oracle(m, t, fi, F, hi, every=np.inf):
    return osolver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, fi, F, [], [], hi, every, 0, "KE",
                                              osolver.VEL_CURRENT)


def test_no_forcing_indices(bfe, plate):
    m = plate
    t = np.arange(40) * m["dt"]
    hi = modelgen.gi_of(m["gl"], m["mon_nds"], 2)
    h, fld, frc, ft = bfe.fn_explicit_dynamic_solver_gb300(m["K"], m["C"], m["M"], t, [], [], [], [], hi, 10, 1,
                                                          "KE", osolver.VEL_CURRENT, "double")
    assert h.shape == (hi.size, 40) and np.all(h == 0)
    assert fld.shape == (m["K"].shape[0], 4) and np.all(fld == 0) and np.all(ft == 0)


@pytest.mark.parametrize("prec", ["double", "single"])
def test_no_monitors_frames_only(bfe, plate, prec):
    m = plate
    t, s = modelgen.pulse(300, m["dt"])
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    _, f0, _, ft0 = _oracle(m, t, fi, s, [], every=75)
    h, f1, _, ft1 = bfe.fn_explicit_dynamic_solver_gb300(m["K"], m["C"], m["M"], t, fi, s, [], [], [], 75, 1, "KE",
                                                         osolver.VEL_CURRENT, prec, gl_lookup=m["gl"])
    assert h is None
    assert _err(f1, f0) <= TOL[prec] and np.array_equal(ft1, ft0)


def test_two_samples_and_a_frame_interval_longer_than_the_run(bfe, plate):
    m = plate
    t = np.arange(2) * m["dt"]
    s = np.array([1.0, -0.5])
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    h0, f0, _, ft0 = _oracle(m, t, fi, s, fi, every=1000)
    h1, f1, _, ft1 = bfe.fn_explicit_dynamic_solver_gb300(m["K"], m["C"], m["M"], t, fi, s, [], [], fi, 1000, 1,
                                                          "KE", osolver.VEL_CURRENT, "double")
    assert f1.shape == f0.shape == (m["K"].shape[0], 1)
    assert _err(h1, h0) <= TOL["double"] and _err(f1, f0) <= TOL["double"] and np.array_equal(ft1, ft0)


@pytest.mark.parametrize("prec,R", [("double", 5), ("single", 5), ("single", 64)])
def test_ragged_sources_with_their_own_signals(bfe, plate, prec, R):
    """Sources with 1, 2 or 3 forced DOFs (padded lists) and one signal row
    per source; R = 64 takes the 64-right-hand-side kernels."""
    m = plate
    nt = 250
    t, s = modelgen.pulse(nt, m["dt"])
    nds = m["mon_nds"]
    srcs = [modelgen.gi_of(m["gl"], nds[(r % 7): (r % 7) + 1 + (r % 3)], 2) for r in range(R)]
    F = np.stack([s[None, :] * (1 + 0.1 * r) for r in range(R)], axis=2)      # (1, nt, R)
    hi = np.concatenate([modelgen.gi_of(m["gl"], nds, 2), srcs[2]])            # includes forced DOFs
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], osolver.VEL_CURRENT, prec, m["gl"]) as plan:
        hb = plan.run_batched(t, srcs, F, hi)
    for r in (0, 2, R - 1):
        h0, _, _, _ = _oracle(m, t, srcs[r], F[:, :, r], hi)
        assert _err(hb[:, :, r], h0) <= TOL[prec], r


def test_repeated_monitors_get_the_same_history(bfe, plate):
    m = plate
    t, s = modelgen.pulse(200, m["dt"])
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    hi = modelgen.gi_of(m["gl"], [m["mon_nds"][3]] * 3 + [m["frc_nd"]], 2)
    h0, _, _, _ = _oracle(m, t, fi, s, hi)
    h1, _, _, _ = bfe.fn_explicit_dynamic_solver_gb300(m["K"], m["C"], m["M"], t, fi, s, [], [], hi, np.inf, 1,
                                                       "KE", osolver.VEL_CURRENT, "double")
    assert np.array_equal(h1[0], h1[1]) and np.array_equal(h1[1], h1[2])
    assert _err(h1, h0) <= TOL["double"]


@pytest.mark.parametrize("prec", ["double", "single"])
def test_one_source_plan(bfe, plate, prec):
    """A plan built with BFE_PLAN_ONE_SOURCE (no batched operator forms)
    gives the one-source results of a full plan bit for bit, and a batched run
    on it (the generic kernel) matches the oracle."""
    m = plate
    t, s = modelgen.pulse(200, m["dt"])
    nds = m["mon_nds"]
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    hi = modelgen.gi_of(m["gl"], nds, 2)
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], osolver.VEL_CURRENT, prec, m["gl"]) as full:
        h_full, f_full, _ = full.run(t, fi, s, hi, 50)
    srcs = [modelgen.gi_of(m["gl"], [nds[r % nds.size]], 1 + r % 2) for r in range(64)]
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], osolver.VEL_CURRENT, prec, m["gl"], one_source=True) as one:
        h_one, f_one, _ = one.run(t, fi, s, hi, 50)
        hb = one.run_batched(t, srcs, s, hi)
        st = one.stats()
    assert np.array_equal(h_one, h_full) and np.array_equal(f_one, f_full)
    assert st["n_groups"] == 0
    for r in (0, 63):
        h0, _, _, _ = _oracle(m, t, srcs[r], s, hi)
        assert _err(hb[:, :, r], h0) <= TOL[prec], r


def test_two_plans_used_concurrently_from_two_threads(bfe, plate):
    """Distinct plans may run at the same time on different host threads
    (the ABI's threading contract): an FP32 64-source run and an FP64
    one-source run started together give the results they give alone."""
    import threading
    m = plate
    t, s = modelgen.pulse(300, m["dt"])
    nds = m["mon_nds"]
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    hi = modelgen.gi_of(m["gl"], nds, 2)
    srcs = [modelgen.gi_of(m["gl"], [nds[r % nds.size]], 1 + r % 2) for r in range(64)]
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], osolver.VEL_CURRENT, "single", m["gl"]) as p32, \
            bfe.Plan(m["K"], m["C"], m["M"], m["dt"], osolver.VEL_CURRENT, "double") as p64:
        alone32 = p32.run_batched(t, srcs, s, hi)
        alone64, _, _ = p64.run(t, fi, s, hi)
        out, errors = {}, []

        def work(name, fn):
            try:
                for k in range(3):
                    out[(name, k)] = fn()
            except Exception as e:          # reported below, on the test's thread
                errors.append(e)
        th = [threading.Thread(target=work, args=("f32", lambda: p32.run_batched(t, srcs, s, hi))),
              threading.Thread(target=work, args=("f64", lambda: p64.run(t, fi, s, hi)[0]))]
        for x in th:
            x.start()
        for x in th:
            x.join()
    assert not errors, errors
    for k in range(3):
        assert np.array_equal(out[("f64", k)], alone64)
        assert _err(out[("f32", k)], alone32) <= 1e-6
