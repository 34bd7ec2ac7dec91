"""The oracle's C port of the v6 loop (oracle/c/cpu_march.c) against the
oracle's NumPy/SciPy restatement (oracle/solver.py): A-scans and field frames
in both solver modes, on a coupled water/steel model with interface rows
(exact P^-1 on the interface block) and absorbers. The C port is the checker
of the full-size GPU tests and the timed CPU baseline, so it must agree with
the restatement to rounding."""
import numpy as np
import pytest

import modelgen
from oracle import cpu_port
from oracle import solver as osolver


@pytest.mark.parametrize("mode", [osolver.VEL_CURRENT, osolver.VEL_LAST_HALF])
@pytest.mark.parametrize("field_type", ["KE", "raw(u)"])
def test_cport_matches_restatement_with_frames(mode, field_type):
    m = modelgen.coupled_model(W=2e-3, Hw=1e-3, Hs=1e-3, h=0.1e-3, abs_thick=0.4e-3)
    nt, every = 260, 50
    t, s = modelgen.pulse(nt, m["dt"])
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 4)
    hi = np.concatenate([modelgen.gi_of(m["gl"], m["mon_nds"], 4), modelgen.gi_of(m["gl"], m["mon_nds"], 2)])
    h0, f0, _, ft0 = osolver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, fi, s, [], [], hi,
                                                        every, 0, field_type, mode)
    op = cpu_port.CpuOperator(m["K"], m["C"], m["M"], m["dt"], mode)
    is_vel = field_type not in osolver.DISP_FIELD_TYPES
    h1, f1, ft1 = op.march(t, fi - 1, s[None, :], hi - 1, every, is_vel, frames=True)
    assert np.abs(h1 - h0).max() <= 1e-12 * np.abs(h0).max()
    assert f1.shape == f0.shape
    assert np.abs(f1 - f0).max() <= 1e-12 * np.abs(f0).max()
    assert np.array_equal(ft1, ft0)
    # without frames the call returns the history alone
    h2 = op.march(t, fi - 1, s[None, :], hi - 1)
    assert np.array_equal(h2, h1)
