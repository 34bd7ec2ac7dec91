"""GPU parity of the v5 scheme (fn_explicit_dynamic_solver_v5.m) through
bfe_run_v5 against the FP64 oracle: forcing, prescribed displacements with
their reaction forces, velocity frames, prescribed DOFs in absorbing layers
and on the fluid-solid interface (rows coupled through off-diagonal C),
repeated prescribed DOFs, forcing shorter than time.

Tolerances: max-normalised error, <= 1e-10 for FP64 plans and <= 1e-4 for
FP32 plans."""
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
    return modelgen.solid_plate(W=4e-3, H=2e-3, h=0.1e-3, dof_to_use=(1, 2), abs_thick=0.8e-3)


@pytest.fixture(scope="module")
def coupled():
    return modelgen.coupled_model(W=3e-3, Hw=1.5e-3, Hs=1.5e-3, h=0.1e-3, abs_thick=0.6e-3, blob=True)


def _compare(res, ref, tol):
    for a, b, name in zip(res, ref, ("history", "field", "force", "field time")):
        if b is None:
            assert a is None, name
            continue
        assert a.shape == b.shape, name
        assert _err(a, b) <= tol, (name, _err(a, b))


@pytest.mark.parametrize("prec", ["double", "single"])
def test_v5_forcing_only_with_frames(bfe, plate, prec):
    m = plate
    t, s = modelgen.pulse(600, m["dt"])
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    hi = modelgen.gi_of(m["gl"], m["mon_nds"], 2)
    ref = osolver.explicit_dynamic_solver_v5(m["K"], m["C"], m["M"], t, fi, s, [], [], hi, 150, 0)
    res = bfe.fn_explicit_dynamic_solver_v5_gb300(m["K"], m["C"], m["M"], t, fi, s, [], [], hi, 150,
                                                  1, prec, gl_lookup=m["gl"])
    _compare(res, ref, TOL[prec])


@pytest.mark.parametrize("prec", ["double", "single"])
@pytest.mark.parametrize("every", [np.inf, 120])
def test_v5_prescribed_displacements_plate(bfe, plate, prec, every):
    """Prescribed vertical displacement at three top-surface nodes (one inside
    the absorbing layer, so C acts on the prescribed DOF), no forcing; the
    march starts at the first non-zero displacement column. Without frames
    the march runs through the CUDA graph."""
    m = plate
    nds = m["mod"]["nds"]
    top = np.nonzero(np.isclose(nds[:, 1], nds[:, 1].max()))[0]
    top = top[np.argsort(nds[top, 0])]
    picks = [top[2], top[top.size // 2], top[top.size // 2 + 3]]
    di = modelgen.gi_of(m["gl"], np.array(picks) + 1, 2)
    t, s = modelgen.pulse(700, m["dt"])
    D = np.vstack([s * 1e-9, 0.5e-9 * s, -0.7e-9 * s])
    D[:, :40] = 0.0
    hi = np.concatenate([modelgen.gi_of(m["gl"], m["mon_nds"], 2), di,
                         modelgen.gi_of(m["gl"], np.array(picks) + 1, 1)])
    ref = osolver.explicit_dynamic_solver_v5(m["K"], m["C"], m["M"], t, [], [], di, D, hi, every, 0)
    res = bfe.fn_explicit_dynamic_solver_v5_gb300(m["K"], m["C"], m["M"], t, [], [], di, D, hi, every,
                                                  1, prec, gl_lookup=m["gl"])
    assert np.abs(ref[2]).max() > 0
    _compare(res, ref, TOL[prec])


@pytest.mark.parametrize("prec", ["double", "single"])
def test_v5_prescribed_on_fluid_solid_interface(bfe, coupled, prec):
    """Prescribed solid DOFs on the interface line: the fluid rows coupled to
    them through ASI2D2's C take the prescribed DOFs' dynamic velocity. Forcing
    in the water as well; monitors on the prescribed DOFs, their fluid
    neighbours and the surface."""
    m = coupled
    nds = m["mod"]["nds"]
    ys = 1.5e-3
    iface = np.nonzero(np.isclose(nds[:, 1], ys))[0]
    iface = iface[np.argsort(nds[iface, 0])]
    mid = iface[iface.size // 2 - 2: iface.size // 2 + 2] + 1
    di = np.concatenate([modelgen.gi_of(m["gl"], mid, 2), modelgen.gi_of(m["gl"], mid[:1], 1)])
    assert di.size == 5
    t, s = modelgen.pulse(800, m["dt"])
    D = np.outer(np.linspace(0.5e-9, 1.5e-9, di.size), s)
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 4)
    hi = np.concatenate([modelgen.gi_of(m["gl"], m["mon_nds"], 4), di, modelgen.gi_of(m["gl"], mid, 4),
                         modelgen.gi_of(m["gl"], iface[::5] + 1, 2)])
    C = m["C"].tocsr()
    coupled_rows = set(np.nonzero(np.asarray(abs(C[:, di - 1]).sum(axis=1)).ravel())[0]) - set(di - 1)
    assert coupled_rows, "no off-diagonal C coupling to the prescribed DOFs"
    ref = osolver.explicit_dynamic_solver_v5(m["K"], m["C"], m["M"], t, fi, s, di, D, hi, 200, 0)
    res = bfe.fn_explicit_dynamic_solver_v5_gb300(m["K"], m["C"], m["M"], t, fi, s, di, D, hi, 200,
                                                  1, prec, gl_lookup=m["gl"])
    _compare(res, ref, TOL[prec])


def test_v5_repeated_prescribed_dofs_and_short_forcing(bfe, plate):
    """Repeated DOF in disp_indices: the last row sets the displacement and
    each force-output row sums the accelerations of every entry of that DOF
    (diag_M(d, d) * accn, v5.m:161). Forcing with fewer columns than time keeps
    its last column (v5.m:145-147); one forcing row broadcasts to two DOFs."""
    m = plate
    t, s = modelgen.pulse(500, m["dt"])
    nds = m["mod"]["nds"]
    top = np.nonzero(np.isclose(nds[:, 1], nds[:, 1].max()))[0]
    top = top[np.argsort(nds[top, 0])]
    a, b = top[top.size // 2 - 4] + 1, top[top.size // 2 + 4] + 1
    di = np.concatenate([modelgen.gi_of(m["gl"], [a], 2), modelgen.gi_of(m["gl"], [b], 2),
                         modelgen.gi_of(m["gl"], [a], 2)])
    D = np.vstack([1e-9 * s, -1e-9 * s, 2e-9 * s])
    fi = np.concatenate([modelgen.gi_of(m["gl"], [m["frc_nd"]], 2), modelgen.gi_of(m["gl"], [m["frc_nd"]], 1)])
    F = s[None, :300] * 1e3
    hi = np.concatenate([modelgen.gi_of(m["gl"], m["mon_nds"], 2), di[:2]])
    ref = osolver.explicit_dynamic_solver_v5(m["K"], m["C"], m["M"], t, fi, F, di, D, hi, np.inf, 0)
    res = bfe.fn_explicit_dynamic_solver_v5_gb300(m["K"], m["C"], m["M"], t, fi, F, di, D, hi, np.inf, 1)
    _compare(res, ref, TOL["double"])
    assert np.allclose(res[0][-2], D[2]), "the last listed row sets a repeated DOF"


def test_v5_matches_v6_last_half_without_prescribed_dofs(bfe, plate):
    """v5.m:150-156 and v6 'vel at last half time step' are the same scheme."""
    m = plate
    t, s = modelgen.pulse(400, m["dt"])
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    hi = modelgen.gi_of(m["gl"], m["mon_nds"], 2)
    h5 = bfe.fn_explicit_dynamic_solver_v5_gb300(m["K"], m["C"], m["M"], t, fi, s, [], [], hi, np.inf)[0]
    h6 = bfe.fn_explicit_dynamic_solver_gb300(m["K"], m["C"], m["M"], t, fi, s, [], [], hi, np.inf, 1,
                                              "KE", osolver.VEL_LAST_HALF, "double")[0]
    assert _err(h5, h6) <= 1e-12


def test_v5_argument_errors(bfe, plate):
    m = plate
    t, s = modelgen.pulse(50, m["dt"])
    di = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], osolver.VEL_LAST_HALF, "double") as p6:
        with pytest.raises(bfe.BfeError, match="BFE_MODE_V5"):
            p6.run_v5(t, [], [], di, s[None, :], [])
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], bfe.V5, "double") as p5:
        two = np.concatenate([di, di + 1])
        with pytest.raises(bfe.BfeError, match="rows"):
            p5.run_v5(t, [], [], two, s[None, :], [])          # one row for two DOFs
        with pytest.raises(bfe.SolverError):
            p5.run_v5(t, [], [], di, s[None, :10], [])         # too few columns
        with pytest.raises(bfe.BfeError, match="out of range"):
            p5.run_v5(t, [], [], [m["K"].shape[0] + 5], s[None, :], [])
