"""Run-time statuses of the C ABI on the GPU: a march that becomes unstable
(time step far above the stability limit) or is fed a non-finite signal
returns BFE_ERR_UNSTABLE with its outputs still written, as the reference
would return them (NaN/Inf values, fn_explicit_dynamic_solver_v6.m:180-218
has no check); a run past the plan's time limit stops between chunks of
steps and returns BFE_ERR_TIMEOUT with the samples computed so far, which
match the oracle; the plan stays usable after either. None of these faults
or hangs the GPU: the statuses are decided on the host."""
import numpy as np
import pytest

import modelgen
from oracle import solver as osolver

pytestmark = pytest.mark.gpu


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
    return modelgen.solid_plate(W=2e-3, H=1e-3, h=0.1e-3)


@pytest.mark.parametrize("prec", ["double", "single"])
@pytest.mark.parametrize("R", [1, 64])
def test_unstable_time_step_returns_unstable(bfe, plate, prec, R):
    from bfe_gb300 import _lib
    m = plate
    dt = 3.0 * m["dt"]                    # the highest mode grows ~30x per step
    nt = 600
    t, s = modelgen.pulse(nt, dt)
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    hi = modelgen.gi_of(m["gl"], m["mon_nds"], 2)
    h0, _, _, _ = osolver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, fi, s, [], [], hi,
                                                     np.inf, 0, "KE", osolver.VEL_CURRENT)
    assert not np.isfinite(h0).all()       # the oracle blows up as well
    with bfe.Plan(m["K"], m["C"], m["M"], dt, bfe.VEL_CURRENT, prec, m["gl"]) as plan:
        with pytest.raises(bfe.BfeError) as ei:
            if R == 1:
                plan.run(t, fi, s, hi)
            else:
                plan.run_batched(t, [fi] * R, s, hi)
        assert ei.value.status == _lib.BFE_ERR_UNSTABLE
        assert "non-finite" in str(ei.value)
        h = ei.value.outputs[0] if R == 1 else ei.value.outputs
        assert not np.isfinite(h).all()    # outputs written as computed


def test_nonfinite_signal_returns_unstable_and_plan_stays_usable(bfe, plate):
    from bfe_gb300 import _lib
    m = plate
    nt = 200
    t, s = modelgen.pulse(nt, m["dt"])
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    hi = modelgen.gi_of(m["gl"], m["mon_nds"], 2)
    bad = s.copy()
    bad[100] = np.nan
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], bfe.VEL_CURRENT, "double") as plan:
        with pytest.raises(bfe.BfeError) as ei:
            plan.run(t, fi, bad, hi)
        assert ei.value.status == _lib.BFE_ERR_UNSTABLE
        h0, _, _, _ = osolver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, fi, s, [], [], hi,
                                                         np.inf, 0, "KE", osolver.VEL_CURRENT)
        h, _, _ = plan.run(t, fi, s, hi)                       # the next run is clean
        assert np.abs(h - h0).max() <= 1e-10 * np.abs(h0).max()


@pytest.mark.parametrize("graph", [True, False])
def test_time_limit_stops_the_run_and_keeps_the_computed_samples(bfe, plate, graph, monkeypatch):
    from bfe_gb300 import _lib
    if not graph:
        monkeypatch.setenv("BFE_NO_GRAPH", "1")
    m = plate
    nt = 6000
    t, s = modelgen.pulse(nt, m["dt"])
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    hi = modelgen.gi_of(m["gl"], m["mon_nds"], 2)
    h0, _, _, _ = osolver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, fi, s, [], [], hi,
                                                     np.inf, 0, "KE", osolver.VEL_CURRENT)
    ti0 = int(np.nonzero(s)[0].min())
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], bfe.VEL_CURRENT, "double") as plan:
        plan.set_time_limit(1e-6)
        with pytest.raises(bfe.BfeError) as ei:
            plan.run(t, fi, s, hi)
        assert ei.value.status == _lib.BFE_ERR_TIMEOUT
        h = ei.value.outputs[0]
        # samples stop at a chunk boundary after the first chunk of 48 steps
        written = np.nonzero(np.abs(h).sum(0))[0]
        last = int(written.max()) + 1
        assert ti0 + 48 <= last < nt
        assert np.abs(h[:, :last] - h0[:, :last]).max() <= 1e-10 * np.abs(h0).max()
        assert np.all(h[:, last + 1:] == 0)
        plan.set_time_limit(0)
        h2, _, _ = plan.run(t, fi, s, hi)                      # no limit: the whole run
        assert np.abs(h2 - h0).max() <= 1e-10 * np.abs(h0).max()
        with pytest.raises(bfe.BfeError) as ei:
            plan.set_time_limit(-1.0)
        assert ei.value.status == _lib.BFE_ERR_ARG
