"""Adjoint gradient (bfe_adjoint_gradient) against the FP64 oracle adjoint and
central finite differences (the acceptance check: 1e-3 relative)."""
import numpy as np
import pytest

import modelgen
from bfe_gb300 import model
from oracle import adjoint as oadj
from oracle import signals

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
def problem():
    """Steel plate with absorbers; observed data from a seeded stiffness
    perturbation (+-5 %); homogeneous candidate model."""
    m = modelgen.solid_plate(W=2e-3, H=1e-3, h=0.1e-3, abs_thick=0.3e-3)
    mod = m["mod"]
    rho = 8000.0
    ed = model.cpe3_element_data(mod["nds"], mod["els"], mod["el_abs_i"], modelgen.STEEL["D"], rho, m["gl"])
    ke, mh, ch, dof = ed
    n = m["K"].shape[0]
    nt = 350
    dt = m["dt"]
    t = np.arange(nt) * dt
    sig = signals.gaussian_pulse(t, 5e6, 5)
    top = m["mon_nds"]
    srcs1 = [modelgen.gi_of(m["gl"], [m["frc_nd"]], 2), modelgen.gi_of(m["gl"], [top[4]], 2)]
    hi1 = modelgen.gi_of(m["gl"], top, 2)
    rng = np.random.default_rng(2)
    s_true = 1 + 0.05 * np.tanh(rng.standard_normal(len(dof)))
    rho_e = np.full(len(dof), rho)
    obs = np.zeros((hi1.size, nt, 2))
    Kt, Ct, Mt = model.assemble_from_elements(ke, mh, ch, dof, n, s_true, rho_e)
    for r, fi in enumerate(srcs1):
        U = oadj.forward(Kt, Mt.diagonal(), Ct.diagonal(), dt, nt, fi - 1, sig[None, :], 0)
        obs[:, :, r] = U[hi1 - 1]
    return dict(m=m, ed=ed, n=n, t=t, dt=dt, sig=sig, srcs1=srcs1, hi1=hi1, obs=obs, rho_e=rho_e)


def _plan(bfe, P, prec, s=None):
    ke, mh, ch, dof = P["ed"]
    K, C, M = model.assemble_from_elements(ke, mh, ch, dof, P["n"], s, P["rho_e"])
    return bfe.Plan(K, C, M, P["dt"], bfe.VEL_CURRENT, prec, P["m"]["gl"])


def _gpu_grad(bfe, P, prec, ckpt=0):
    ke, mh, ch, dof = P["ed"]
    with _plan(bfe, P, prec) as plan:
        return plan.adjoint_gradient((ke, mh, ch, dof), P["t"], P["srcs1"], P["sig"], P["hi1"],
                                     P["obs"], ckpt_every=ckpt)


def test_fp64_adjoint_matches_oracle_adjoint(bfe, problem):
    P = problem
    ke, mh, ch, dof = P["ed"]
    J0, gs0, gr0 = oadj.misfit_and_gradient(ke, mh, ch, dof, P["n"], P["dt"], P["t"].size,
                                            [s - 1 for s in P["srcs1"]], P["sig"][None, :],
                                            P["hi1"] - 1, P["obs"], rho_e=P["rho_e"])
    J1, gs1, gr1 = _gpu_grad(bfe, P, "double")
    assert abs(J1 - J0) <= 1e-9 * J0
    assert np.abs(gs1 - gs0).max() <= 1e-8 * np.abs(gs0).max()
    assert np.abs(gr1 - gr0).max() <= 1e-8 * np.abs(gr0).max()


def test_adjoint_matches_central_finite_differences(bfe, problem):
    P = problem
    J, gs, gr = _gpu_grad(bfe, P, "double")
    ke, mh, ch, dof = P["ed"]
    rng = np.random.default_rng(3)
    big = np.argsort(-np.abs(gs))[:200]             # elements the A-scans are sensitive to
    picks = rng.choice(big, 6, replace=False)

    def J_at(s=None, rho=None):
        K, C, M = model.assemble_from_elements(ke, mh, ch, dof, P["n"], s,
                                               P["rho_e"] if rho is None else rho)
        with bfe.Plan(K, C, M, P["dt"], bfe.VEL_CURRENT, "double") as plan:
            h = plan.run_batched(P["t"], P["srcs1"], P["sig"], P["hi1"])
        return 0.5 * ((h - P["obs"]) ** 2).sum()
    for e in picks:
        eps = 1e-3
        sp_, sm_ = np.ones(len(dof)), np.ones(len(dof))
        sp_[e] += eps
        sm_[e] -= eps
        fd = (J_at(s=sp_) - J_at(s=sm_)) / (2 * eps)
        assert abs(gs[e] - fd) <= 1e-3 * abs(fd), (e, gs[e], fd)
        rp, rm = P["rho_e"].copy(), P["rho_e"].copy()
        rp[e] *= 1 + eps
        rm[e] *= 1 - eps
        fdr = (J_at(rho=rp) - J_at(rho=rm)) / (2 * eps * P["rho_e"][e])
        assert abs(gr[e] - fdr) <= 1e-3 * abs(fdr), (e, gr[e], fdr)


@pytest.mark.parametrize("prec,tol", [("double", 1e-12), ("single", 1e-5)])
def test_checkpoint_interval_does_not_change_gradient(bfe, problem, prec, tol):
    """ckpt_every = 0 keeps every forward state on the device (this model is
    small); 1, 13 and n_t recompute segments from checkpoints. The gradients
    differ only by the order of the per-segment sums."""
    b = _gpu_grad(bfe, problem, prec, ckpt=0)
    for ck in (1, 13, problem["t"].size):
        x = _gpu_grad(bfe, problem, prec, ckpt=ck)
        assert x[0] == pytest.approx(b[0], rel=tol)
        assert np.abs(x[1] - b[1]).max() <= tol * np.abs(b[1]).max()
        assert np.abs(x[2] - b[2]).max() <= tol * np.abs(b[2]).max()


def test_fp32_adjoint_close_to_fp64(bfe, problem):
    J64, gs64, gr64 = _gpu_grad(bfe, problem, "double")
    J32, gs32, gr32 = _gpu_grad(bfe, problem, "single")
    assert abs(J32 - J64) <= 1e-3 * J64
    assert np.linalg.norm(gs32 - gs64) <= 1e-3 * np.linalg.norm(gs64)
    assert np.linalg.norm(gr32 - gr64) <= 1e-3 * np.linalg.norm(gr64)


def test_autograd_wrapper_gradient(bfe, problem):
    import torch
    from bfe_gb300.autograd import AscanMisfit
    P = problem
    ne = len(P["ed"][3])
    prob = dict(element_data=P["ed"], n=P["n"], dt=P["dt"], time=P["t"], sources=P["srcs1"],
                signal=P["sig"], monitors=P["hi1"], observed=P["obs"], gl_lookup=P["m"]["gl"])
    s = torch.ones(ne, dtype=torch.float64, requires_grad=True)
    rho = torch.tensor(P["rho_e"], requires_grad=True)
    J = AscanMisfit.apply(s, rho, prob)
    J.backward()
    J_ref, gs, gr = _gpu_grad(bfe, P, "double")
    assert float(J.detach()) == pytest.approx(J_ref, rel=1e-12)
    assert np.allclose(s.grad.numpy(), gs, rtol=1e-10, atol=1e-30)
    assert np.allclose(rho.grad.numpy(), gr, rtol=1e-10, atol=1e-40)


def test_fp32_adjoint_with_16_sources_matches_fp64(bfe, problem):
    """16 sources take the 4-lanes-per-node FP32 kernels in the forward,
    recompute and adjoint marches; FP32 and FP64 gradients agree."""
    P = problem
    ke, mh, ch, dof = P["ed"]
    top = P["m"]["mon_nds"]
    srcs = [modelgen.gi_of(P["m"]["gl"], [top[k % top.size]], 1 + (k // top.size) % 2) for k in range(16)]
    obs = np.zeros((P["hi1"].size, P["t"].size, 16))
    obs[:, :, :2] = P["obs"]
    out = {}
    for prec in ("double", "single"):
        with _plan(bfe, P, prec) as plan:
            out[prec] = plan.adjoint_gradient((ke, mh, ch, dof), P["t"], srcs, P["sig"], P["hi1"], obs)
    (J64, gs64, gr64), (J32, gs32, gr32) = out["double"], out["single"]
    assert abs(J32 - J64) <= 1e-4 * J64
    assert np.linalg.norm(gs32 - gs64) <= 1e-4 * np.linalg.norm(gs64)
    assert np.linalg.norm(gr32 - gr64) <= 1e-4 * np.linalg.norm(gr64)


@pytest.mark.parametrize("R", [1, 16])
def test_fp64_adjoint_with_1_or_16_sources_matches_oracle(bfe, problem, R):
    """16 sources: the FP64 contraction reads two sources per 16-byte load
    with eight lanes per element; every source's gradient adds up as the
    oracle's per-source sum. One source: the one-source march kernels and a
    lane per element."""
    P = problem
    ke, mh, ch, dof = P["ed"]
    top = P["m"]["mon_nds"]
    srcs = [modelgen.gi_of(P["m"]["gl"], [top[k % top.size]], 1 + (k // top.size) % 2) for k in range(R)]
    rng = np.random.default_rng(5)
    obs = 1e-3 * rng.standard_normal((P["hi1"].size, P["t"].size, R)) * np.abs(P["obs"]).max()
    J0, gs0, gr0 = oadj.misfit_and_gradient(ke, mh, ch, dof, P["n"], P["dt"], P["t"].size,
                                            [s - 1 for s in srcs], P["sig"][None, :], P["hi1"] - 1, obs,
                                            rho_e=P["rho_e"])
    with _plan(bfe, P, "double") as plan:
        J1, gs1, gr1 = plan.adjoint_gradient((ke, mh, ch, dof), P["t"], srcs, P["sig"], P["hi1"], obs,
                                             ckpt_every=7)
    assert abs(J1 - J0) <= 1e-9 * J0
    assert np.abs(gs1 - gs0).max() <= 1e-8 * np.abs(gs0).max()
    assert np.abs(gr1 - gr0).max() <= 1e-8 * np.abs(gr0).max()


@pytest.mark.parametrize("prec,tol", [("double", 1e-8), ("single", 1e-3)])
def test_brick_adjoint_matches_oracle(bfe, prec, tol):
    """3D 8-node bricks (24 DOFs per element) with damped elements, 4 sources
    normal to the top face: FP64 and FP32 gradients against the oracle."""
    nds, els, n3, d = model.cubic_mesh(0.6e-3, 0.6e-3, 0.3e-3, 0.1e-3)
    rho = model.STEEL["rho"]
    D = model.isotropic_stiffness(model.STEEL["E"], model.STEEL["nu"])
    kb, me = model.brick_matrices(d[0], d[1], d[2], D, rho)
    ne = els.shape[0]
    rng = np.random.default_rng(7)
    a = np.where(rng.random(ne) < 0.3, rng.random(ne), 0.0)
    ke = np.repeat(kb[None], ne, axis=0) * np.exp(np.log(0.01) * a ** 4)[:, None, None]
    mh = np.full((ne, 24), me / rho)
    ch = mh * (a ** 3 * 3.1415e7)[:, None]
    dof = (3 * (els[:, :, None] - 1) + np.arange(3)[None, None, :]).reshape(ne, 24)
    n = 3 * nds.shape[0]
    gl = (3 * np.arange(nds.shape[0])[:, None] + np.arange(3)[None, :] + 1).astype(np.int64)
    dt = 0.9 * 2.0 / np.sqrt(np.linalg.eigvalsh(kb / me).max())
    nt = 160
    t = np.arange(nt) * dt
    sig = signals.gaussian_pulse(t, 5e6, 5)
    top = np.nonzero(np.isclose(nds[:, 2], nds[:, 2].max()))[0]
    srcs = [np.array([3 * top[k] + 3]) for k in (0, 8, 17, 30)]
    hi = 3 * top[::3] + 3
    rho_e = np.full(ne, rho)
    s_true = 1 + 0.05 * np.tanh(rng.standard_normal(ne))
    Kt, Ct, Mt = model.assemble_from_elements(ke, mh, ch, dof, n, s_true, rho_e)
    obs = np.zeros((hi.size, nt, len(srcs)))
    for r, fi in enumerate(srcs):
        obs[:, :, r] = oadj.forward(Kt, Mt.diagonal(), Ct.diagonal(), dt, nt, fi - 1, sig[None, :], 0)[hi - 1]
    J0, gs0, gr0 = oadj.misfit_and_gradient(ke, mh, ch, dof, n, dt, nt, [s - 1 for s in srcs], sig[None, :],
                                            hi - 1, obs, rho_e=rho_e)
    K, C, M = model.assemble_from_elements(ke, mh, ch, dof, n, None, rho_e)
    with bfe.Plan(K, C, M, dt, bfe.VEL_CURRENT, prec, gl) as plan:
        J1, gs1, gr1 = plan.adjoint_gradient((ke, mh, ch, dof), t, srcs, sig, hi, obs)
    assert abs(J1 - J0) <= tol * J0
    assert np.abs(gs1 - gs0).max() <= tol * np.abs(gs0).max()
    assert np.abs(gr1 - gr0).max() <= tol * np.abs(gr0).max()


@pytest.mark.parametrize("prec,tol", [("double", 1e-8), ("single", 1e-3)])
def test_unused_element_dofs_with_16_sources_match_oracle(bfe, problem, prec, tol):
    """Element DOF entries of -1 (unused) with 16 sources: the contraction
    reads row 0 for them (FP32: unmasked, the factor's row is zero) or masks
    them (FP64). The oracle gets the same model written with a valid index
    there and that entry's K_e row and column, Mh and Ch zeroed."""
    P = problem
    ke, mh, ch, dof = P["ed"]
    ne = len(dof)
    pick = np.arange(0, ne, 37)
    col = pick % dof.shape[1]
    dof_u = dof.copy()
    dof_u[pick, col] = -1
    ke_o, mh_o, ch_o, dof_o = ke.copy(), mh.copy(), ch.copy(), dof.copy()
    ke_o[pick, col, :] = 0.0
    ke_o[pick, :, col] = 0.0
    mh_o[pick, col] = 0.0
    ch_o[pick, col] = 0.0
    dof_o[pick, col] = 0
    top = P["m"]["mon_nds"]
    srcs = [modelgen.gi_of(P["m"]["gl"], [top[k % top.size]], 1 + (k // top.size) % 2) for k in range(16)]
    rng = np.random.default_rng(11)
    obs = 1e-3 * rng.standard_normal((P["hi1"].size, P["t"].size, 16)) * np.abs(P["obs"]).max()
    J0, gs0, gr0 = oadj.misfit_and_gradient(ke_o, mh_o, ch_o, dof_o, P["n"], P["dt"], P["t"].size,
                                            [s - 1 for s in srcs], P["sig"][None, :], P["hi1"] - 1, obs,
                                            rho_e=P["rho_e"])
    K, C, M = model.assemble_from_elements(ke_o, mh_o, ch_o, dof_o, P["n"], None, P["rho_e"])
    with bfe.Plan(K, C, M, P["dt"], bfe.VEL_CURRENT, prec, P["m"]["gl"]) as plan:
        J1, gs1, gr1 = plan.adjoint_gradient((ke, mh, ch, dof_u), P["t"], srcs, P["sig"], P["hi1"], obs)
    assert abs(J1 - J0) <= tol * J0
    assert np.abs(gs1 - gs0).max() <= tol * np.abs(gs0).max()
    assert np.abs(gr1 - gr0).max() <= tol * np.abs(gr0).max()


@pytest.mark.parametrize("prec,R,tol", [("double", 2, 1e-8), ("double", 16, 1e-8), ("single", 16, 1e-3)])
def test_three_dof_cpe3_adjoint_matches_oracle(bfe, prec, R, tol):
    """CPE3 with DOFs 1, 2 and 3 (9 DOFs per element, out-of-plane motion
    included) and an absorbing layer: gradients against the oracle."""
    m = modelgen.solid_plate(W=2e-3, H=1e-3, h=0.1e-3, dof_to_use=(1, 2, 3), abs_thick=0.3e-3)
    mod = m["mod"]
    rho = 8000.0
    ke, mh, ch, dof = model.cpe3_element_data(mod["nds"], mod["els"], mod["el_abs_i"], modelgen.STEEL["D"], rho,
                                              m["gl"], dof_to_use=(1, 2, 3))
    assert dof.shape[1] == 9
    n = m["K"].shape[0]
    nt = 250
    t = np.arange(nt) * m["dt"]
    sig = signals.gaussian_pulse(t, 5e6, 5)
    top = m["mon_nds"]
    srcs = [modelgen.gi_of(m["gl"], [top[(5 * k) % top.size]], 1 + k % 3) for k in range(R)]
    hi = np.concatenate([modelgen.gi_of(m["gl"], top, 2), modelgen.gi_of(m["gl"], top, 3)])
    rho_e = np.full(len(dof), rho)
    rng = np.random.default_rng(11)
    s_true = 1 + 0.05 * np.tanh(rng.standard_normal(len(dof)))
    Kt, Ct, Mt = model.assemble_from_elements(ke, mh, ch, dof, n, s_true, rho_e)
    obs = np.zeros((hi.size, nt, R))
    for r, fi in enumerate(srcs):
        obs[:, :, r] = oadj.forward(Kt, Mt.diagonal(), Ct.diagonal(), m["dt"], nt, fi - 1, sig[None, :], 0)[hi - 1]
    J0, gs0, gr0 = oadj.misfit_and_gradient(ke, mh, ch, dof, n, m["dt"], nt, [s - 1 for s in srcs], sig[None, :],
                                            hi - 1, obs, rho_e=rho_e)
    K, C, M = model.assemble_from_elements(ke, mh, ch, dof, n, None, rho_e)
    with bfe.Plan(K, C, M, m["dt"], bfe.VEL_CURRENT, prec, m["gl"]) as plan:
        J1, gs1, gr1 = plan.adjoint_gradient((ke, mh, ch, dof), t, srcs, sig, hi, obs)
    assert abs(J1 - J0) <= tol * J0
    assert np.abs(gs1 - gs0).max() <= tol * np.abs(gs0).max()
    assert np.abs(gr1 - gr0).max() <= tol * np.abs(gr0).max()


@pytest.mark.parametrize("prec,R,tol", [("double", 4, 1e-8), ("single", 16, 1e-3), ("single", 1, 1e-3)])
def test_one_dof_triangle_adjoint_matches_oracle(bfe, prec, R, tol):
    """Scalar waves on linear triangles (one DOF per node, 3 per element, the
    fluid element's layout), bulk modulus 2.2 GPa, density 1000, damped
    absorber elements: gradients against the oracle."""
    m = modelgen.solid_plate(W=2e-3, H=1e-3, h=0.1e-3, abs_thick=0.3e-3)
    mod = m["mod"]
    nds, els = mod["nds"], mod["els"][:, :3] - 1
    x, y = nds[els, 0], nds[els, 1]
    det = (x[:, 1] - x[:, 0]) * (y[:, 2] - y[:, 0]) - (x[:, 2] - x[:, 0]) * (y[:, 1] - y[:, 0])
    area = 0.5 * np.abs(det)
    b = np.stack([y[:, 1] - y[:, 2], y[:, 2] - y[:, 0], y[:, 0] - y[:, 1]], 1) / det[:, None]
    c = np.stack([x[:, 2] - x[:, 1], x[:, 0] - x[:, 2], x[:, 1] - x[:, 0]], 1) / det[:, None]
    a = np.asarray(mod["el_abs_i"], float)
    ke = 2.2e9 * area[:, None, None] * (b[:, :, None] * b[:, None, :] + c[:, :, None] * c[:, None, :])
    ke *= np.exp(np.log(0.01) * a ** 4)[:, None, None]
    mh = np.repeat(area[:, None] / 3, 3, axis=1)
    ch = mh * (a ** 3 * 3.1415e7)[:, None]
    dof = els.astype(np.int64)
    n = nds.shape[0]
    rho = 1000.0
    lam = max(np.linalg.eigvalsh(ke[e] / (rho * mh[e][:, None])).max() for e in range(0, len(dof), 7))
    dt = 0.8 * 2.0 / np.sqrt(lam)
    nt = 250
    t = np.arange(nt) * dt
    sig = signals.gaussian_pulse(t, 2e6, 5)
    top = m["mon_nds"] - 1
    srcs = [np.array([top[(3 * k) % top.size] + 1]) for k in range(R)]
    hi = top[::2] + 1
    rho_e = np.full(len(dof), rho)
    rng = np.random.default_rng(13)
    s_true = 1 + 0.05 * np.tanh(rng.standard_normal(len(dof)))
    Kt, Ct, Mt = model.assemble_from_elements(ke, mh, ch, dof, n, s_true, rho_e)
    obs = np.zeros((hi.size, nt, R))
    for r, fi in enumerate(srcs):
        obs[:, :, r] = oadj.forward(Kt, Mt.diagonal(), Ct.diagonal(), dt, nt, fi - 1, sig[None, :], 0)[hi - 1]
    J0, gs0, gr0 = oadj.misfit_and_gradient(ke, mh, ch, dof, n, dt, nt, [s - 1 for s in srcs], sig[None, :],
                                            hi - 1, obs, rho_e=rho_e)
    assert J0 > 0 and np.abs(gs0).max() > 0
    K, C, M = model.assemble_from_elements(ke, mh, ch, dof, n, None, rho_e)
    with bfe.Plan(K, C, M, dt, bfe.VEL_CURRENT, prec) as plan:
        J1, gs1, gr1 = plan.adjoint_gradient((ke, mh, ch, dof), t, srcs, sig, hi, obs)
    assert abs(J1 - J0) <= tol * J0
    assert np.abs(gs1 - gs0).max() <= tol * np.abs(gs0).max()
    assert np.abs(gr1 - gr0).max() <= tol * np.abs(gr0).max()


def test_plans_with_fluid_solid_interface_rows_are_rejected(bfe):
    """A coupled water/steel plan: ASI2D2 puts the fluid-solid coupling in C
    (fn_el_ASI2D2.m:61-76), so P is not diagonal on the interface rows and
    the adjoint returns BFE_ERR_UNSUPPORTED instead of a wrong gradient."""
    from bfe_gb300 import _lib
    m = modelgen.coupled_model(W=2e-3, Hw=1e-3, Hs=1e-3, h=0.1e-3, abs_thick=0.3e-3)
    n = m["K"].shape[0]
    nt = 60
    t = np.arange(nt) * m["dt"]
    sig = signals.gaussian_pulse(t, 5e6, 5)
    src = [modelgen.gi_of(m["gl"], [m["frc_nd"]], 4)]
    hi = modelgen.gi_of(m["gl"], m["mon_nds"], 4)
    dof = np.arange(3 * (n // 3), dtype=np.int64).reshape(-1, 3)
    ke = np.zeros((dof.shape[0], 3, 3))
    mh = np.ones((dof.shape[0], 3))
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], bfe.VEL_CURRENT, "double") as plan:
        with pytest.raises(bfe.BfeError) as ei:
            plan.adjoint_gradient((ke, mh, 0 * mh, dof), t, src, sig, hi, np.zeros((hi.size, nt, 1)))
    assert ei.value.status == _lib.BFE_ERR_UNSUPPORTED
    assert "interface" in str(ei.value)
