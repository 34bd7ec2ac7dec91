"""GPU parity of the element field output (fn_get_field_output.m) and of the
entry function mirror (fn_BristolFE_v2.m) against the FP64 oracle.

Tolerances: max-normalised error, <= 1e-12 for the field reduction of given
frames, <= 1e-10 for FP64 marches, <= 1e-4 for FP32 marches."""
import numpy as np
import pytest

import modelgen
from oracle import entry as oentry
from oracle import solver as osolver

pytestmark = pytest.mark.gpu

FIELD_TYPES = ["sqrt(KE)", "KE", "mean(u1)", "mean(v2)", "div(u)", "curl(v)"]


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
def coupled():
    return modelgen.coupled_model(W=3e-3, Hw=1.5e-3, Hs=1.5e-3, h=0.1e-3, abs_thick=0.6e-3, blob=True)


def _mats(m):
    return dict(K=m["K"], C=m["C"], M=m["M"], gl_lookup=m["gl"])


@pytest.mark.parametrize("ftype", FIELD_TYPES)
def test_field_output_of_given_frames(bfe, coupled, ftype):
    m = coupled
    f = np.random.default_rng(5).standard_normal((m["K"].shape[0], 4))
    ref = oentry.get_field_output(f, m["mod"], _mats(m), ftype)
    got = bfe.fn_get_field_output_gb300(f, m["mod"], _mats(m), ftype)
    assert got.shape == ref.shape
    assert _err(got, ref) <= 1e-12


def test_raw_field_type_returns_the_type_string(bfe, coupled):
    f = np.zeros((coupled["K"].shape[0], 2))
    assert bfe.fn_get_field_output_gb300(f, coupled["mod"], _mats(coupled), "raw(v)") == "raw(v)"


def test_curl_is_rejected_for_3d(bfe):
    from bfe_gb300 import FieldOutput
    nds = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1.0]])
    els = np.array([[1, 2, 3, 4]])
    gl = np.arange(1, 13).reshape(4, 3)
    import scipy.sparse as sp
    with pytest.raises(bfe.BfeError, match="curl"):
        FieldOutput(nds, els, gl, sp.identity(12, format="csr"), "curl(u)")


@pytest.mark.parametrize("prec,tol", [("double", 1e-10), ("single", 1e-4)])
@pytest.mark.parametrize("ftype", ["KE", "mean(u2)", "div(v)"])
def test_run_reduces_frames_on_device(bfe, coupled, prec, tol, ftype):
    """bfe_run_field: frames are reduced as the march produces them."""
    m = coupled
    t, s = modelgen.pulse(600, m["dt"])
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 4)
    hi = modelgen.gi_of(m["gl"], m["mon_nds"], 4)
    h0, f0, _, ft0 = osolver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, fi, s, [], [], hi, 150, 0,
                                                        ftype, osolver.VEL_CURRENT)
    ref = oentry.get_field_output(f0, m["mod"], _mats(m), ftype)
    is_vel = ftype not in ("mean(u1)", "mean(u2)", "mean(u3)", "curl(u)", "div(u)", "raw(u)")
    with bfe.FieldOutput(m["mod"]["nds"], m["mod"]["els"], m["gl"], m["M"], ftype) as fo, \
            bfe.Plan(m["K"], m["C"], m["M"], m["dt"], osolver.VEL_CURRENT, prec, m["gl"]) as plan:
        h1, el, ft1 = plan.run(t, fi, s, hi, 150, is_vel, field=fo)
    assert el.shape == ref.shape
    assert _err(h1, h0) <= tol
    assert _err(el, ref) <= tol
    assert np.array_equal(ft1, ft0)


def _steps(m, t, s, n_src=3, with_frames_nodes=False):
    nds = m["mod"]["nds"]
    top = np.nonzero(np.isclose(nds[:, 1], nds[:, 1].max()))[0]
    top = top[np.argsort(nds[top, 0])]
    src = top[np.linspace(top.size // 4, 3 * top.size // 4, n_src).astype(int)] + 1
    mon_nds = np.concatenate([m["mon_nds"], [m["mon_nds"][0]]])
    mon_dfs = np.full(mon_nds.size, 4)
    mon_dfs[-1] = 1                         # no DOF 1 on a water node: dropped, res.dsps keeps a row
    steps = []
    for k, sn in enumerate(src):
        steps.append(dict(load=dict(time=t, frcs=s[None, :] * (1 + k), frc_nds=[sn], frc_dfs=[4]),
                          mon=dict(nds=mon_nds, dfs=mon_dfs)))
    return steps


@pytest.mark.parametrize("batch", [True, False])
def test_entry_matches_oracle_entry_batched_steps(bfe, coupled, batch):
    """Three transmitter steps with the same monitors: one multi-RHS march
    (batch_steps) or three single marches, both equal to the oracle's
    fn_BristolFE_v2 step loop."""
    from bfe_gb300.entry import fn_BristolFE_v2_gb300
    m = coupled
    t, s = modelgen.pulse(500, m["dt"])
    steps = _steps(m, t, s)
    opts = dict(dof_to_use=[1, 2, 4], damping_power_law=2, batch_steps=batch)
    ref, rmats = oentry.BristolFE_v2(m["mod"], m["matls"], steps, dict(opts))
    got, gmats = fn_BristolFE_v2_gb300(m["mod"], m["matls"], steps, dict(opts))
    assert np.array_equal(gmats["gl_lookup"], rmats["gl_lookup"])
    assert len(got) == len(ref) == 3
    for g, r in zip(got, ref):
        assert np.array_equal(g["valid_mon_dsps"], r["valid_mon_dsps"])
        assert np.array_equal(g["dsp_gi"], r["dsp_gi"])
        assert g["dsps"].shape == r["dsps"].shape
        assert _err(g["dsps"], r["dsps"]) <= 1e-10
        assert g["fld"] is None and g["frcs"] is None


def test_entry_with_field_output_and_wts(bfe, coupled):
    """Frames every 100 samples reduced to sqrt(KE) per element on the device,
    steps{1}.load.wts applied to every step's forces (fn_BristolFE_v2.m:79)."""
    from bfe_gb300.entry import fn_BristolFE_v2_gb300
    m = coupled
    t, s = modelgen.pulse(400, m["dt"])
    steps = _steps(m, t, s, n_src=2)
    steps[0]["load"]["wts"] = [0.5]
    opts = dict(dof_to_use=[1, 2, 4], damping_power_law=2, field_output_every_n_frames=100,
                field_output_type="KE")
    ref, _ = oentry.BristolFE_v2(m["mod"], m["matls"], steps, dict(opts))
    got, _ = fn_BristolFE_v2_gb300(m["mod"], m["matls"], steps, dict(opts))
    for g, r in zip(got, ref):
        assert _err(g["dsps"], r["dsps"]) <= 1e-10
        assert _err(g["fld"], r["fld"]) <= 1e-10
        assert np.array_equal(g["fld_time"], r["fld_time"])


def test_entry_v5_with_prescribed_displacements(bfe, coupled):
    """dynamic_solver_version 'v5': prescribed displacements on the interface
    and their reaction forces (res.frcs), velocity frames as mean(v2)."""
    from bfe_gb300.entry import fn_BristolFE_v2_gb300
    m = coupled
    t, s = modelgen.pulse(400, m["dt"])
    nds = m["mod"]["nds"]
    iface = np.nonzero(np.isclose(nds[:, 1], 1.5e-3))[0]
    iface = iface[np.argsort(nds[iface, 0])]
    dn = iface[iface.size // 2 - 1: iface.size // 2 + 2] + 1
    steps = [dict(load=dict(time=t, dsps=np.outer([1e-9, 2e-9, 3e-9, 1e-9], s),
                            dsp_nds=np.concatenate([dn, dn[:1]]), dsp_dfs=[2, 2, 2, 4]),
                  mon=dict(nds=m["mon_nds"], dfs=np.full(len(m["mon_nds"]), 4)))]
    opts = dict(dof_to_use=[1, 2, 4], damping_power_law=2, dynamic_solver_version="v5",
                field_output_every_n_frames=100, field_output_type="mean(v2)")
    ref, _ = oentry.BristolFE_v2(m["mod"], m["matls"], steps, dict(opts))
    got, _ = fn_BristolFE_v2_gb300(m["mod"], m["matls"], steps, dict(opts))
    g, r = got[0], ref[0]
    assert np.array_equal(g["valid_appl_dsps"], r["valid_appl_dsps"])
    assert _err(g["dsps"], r["dsps"]) <= 1e-10
    assert g["frcs"].shape == r["frcs"].shape
    assert _err(g["frcs"], r["frcs"]) <= 1e-10
    assert _err(g["fld"], r["fld"]) <= 1e-10


def test_entry_options_only_and_raw_type(bfe, coupled):
    from bfe_gb300.entry import fn_BristolFE_v2_gb300
    m = coupled
    opts = fn_BristolFE_v2_gb300(m["mod"], m["matls"], [], {})
    assert opts["dynamic_solver_version"] == "v6" and opts["solver_mode"] == osolver.VEL_CURRENT
    t, s = modelgen.pulse(200, m["dt"])
    steps = _steps(m, t, s, n_src=1)
    opts = dict(dof_to_use=[1, 2, 4], damping_power_law=2, field_output_every_n_frames=50,
                field_output_type="raw(u)")
    got, _ = fn_BristolFE_v2_gb300(m["mod"], m["matls"], steps, opts)
    assert got[0]["fld"] == "raw(u)"
    assert got[0]["fld_time"].shape == (4,)
