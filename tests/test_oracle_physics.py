"""Known-answer checks that pin the oracle's assembly and time marching, taken
from the reference's own test scripts (tests/stability.m,
tests/fn_amplification_matrix.m, tests/fn_fluid_solid.m) and FE identities."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import assembly, entry, mesh, signals, solver
import modelgen


def test_c0_shape_and_nnz():
    # 20 x 10 mm at 0.1 mm: 201 x 101 nodes, 40,000 CPE3, 40,602 DOF, nnz 483,600
    m = modelgen.solid_plate(W=20e-3, H=10e-3, h=0.1e-3)
    assert m["mod"]["nds"].shape[0] == 20301
    assert m["mod"]["els"].shape[0] == 40000
    assert m["K"].shape == (40602, 40602)
    assert m["K"].nnz == 483600


def test_dof_numbering_node_major_dof_minor():
    # gi = (nd - 1) * max_df + df, compacted (fn_build_global_matrices_v5.m:127-159)
    m = modelgen.solid_plate(W=0.3e-3, H=0.2e-3, h=0.1e-3)
    gl = m["gl"]
    n_nodes = m["mod"]["nds"].shape[0]
    assert gl.shape == (n_nodes, 2)
    assert np.array_equal(gl.ravel(), np.arange(1, 2 * n_nodes + 1))


def test_dof_numbering_with_fluid_compacts_unused():
    m = modelgen.coupled_model(W=1e-3, Hw=0.5e-3, Hs=0.5e-3, h=0.1e-3, abs_thick=0)
    gl = m["gl"]
    assert gl.shape[1] == 4                 # max_df = 4 with fluid present
    assert np.all(gl[:, 2] == 0)            # DOF 3 not used with dof_to_use [1 2 4]
    used = np.sort(gl[gl > 0])
    assert np.array_equal(used, np.arange(1, used.size + 1))
    # numbering increases node-major then dof-minor
    order = [(a, d) for a in range(gl.shape[0]) for d in range(gl.shape[1]) if gl[a, d] > 0]
    assert [gl[a, d] for a, d in order] == list(range(1, used.size + 1))


def test_stiffness_symmetric_and_rigid_translation_free():
    m = modelgen.solid_plate(W=2e-3, H=1e-3, h=0.1e-3)
    K = m["K"]
    assert abs(K - K.T).max() <= 1e-12 * abs(K).max()
    n = K.shape[0]
    tx = np.zeros(n); tx[0::2] = 1
    ty = np.zeros(n); ty[1::2] = 1
    assert np.abs(K @ tx).max() <= 1e-9 * abs(K).max()
    assert np.abs(K @ ty).max() <= 1e-9 * abs(K).max()


def test_lumped_mass_total():
    W, H = 2e-3, 1e-3
    m = modelgen.solid_plate(W=W, H=H, h=0.1e-3)
    assert np.isclose(m["M"].sum() / 2, 8000 * W * H, rtol=1e-12)


def test_amplification_matrix_stability_threshold():
    # tests/stability.m:61-71: spectral radius <= 1 below the critical dt, > 1 above
    matls = [dict(modelgen.STEEL)]
    nds = np.array([[0.5, np.sqrt(3) / 2], [0, 0], [1, 0]]) * 1e-3
    els = np.array([[1, 2, 3]])
    K, C, M, _ = assembly.build_global_matrices_v5(nds, els, [1], [0], ["CPE3"], matls, {})
    dt_stable = signals.element_eigen_time_step(nds, els, matls[0]["D"], matls[0]["rho"], factor=0.99)
    # rigid-body modes give a defective eigenvalue 1, which dense eig resolves
    # only to ~sqrt(eps)
    assert solver.amplification_matrix_max_ev(M, C, K, dt_stable) <= 1 + 1e-6
    assert solver.amplification_matrix_max_ev(M, C, K, dt_stable * 1.05) > 1 + 1e-3
    assert solver.amplification_matrix_max_ev(M, C, K, dt_stable, solver.VEL_CURRENT) <= 1 + 1e-6


def test_v5_equals_v6_last_half_step():
    # The two central-difference forms are algebraically identical (v5.m:150-156
    # vs v6.m:131-134), so their histories agree to rounding.
    m = modelgen.solid_plate(W=2e-3, H=1e-3, h=0.1e-3, abs_thick=0.3e-3)
    nt = 300
    t, s = modelgen.pulse(nt, m["dt"])
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    hi = modelgen.gi_of(m["gl"], m["mon_nds"], 2)
    h6, _, _, _ = solver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, fi, s, [], [], hi,
                                                    np.inf, 0, "KE", solver.VEL_LAST_HALF)
    h5, _, _, _ = solver.explicit_dynamic_solver_v5(m["K"], m["C"], m["M"], t, fi, s, [], [], hi, np.inf, 0)
    assert np.abs(h5 - h6).max() <= 1e-9 * np.abs(h6).max()


def test_v5_prescribing_the_forced_displacement_reproduces_the_run():
    # v5.m:150-162: prescribing at the forced DOF the displacement history of a
    # forced run leaves every other DOF's history unchanged (C = 0 there), and
    # the reaction force m accn + K(d,:) u_previous equals the applied force,
    # since accn is the scheme's own second difference (v5.m:73-76).
    m = modelgen.solid_plate(W=2e-3, H=1e-3, h=0.1e-3)
    nt = 300
    t, s = modelgen.pulse(nt, m["dt"])
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    hi = np.concatenate([modelgen.gi_of(m["gl"], m["mon_nds"], 2), fi])
    h1, _, f1, _ = solver.explicit_dynamic_solver_v5(m["K"], m["C"], m["M"], t, fi, s, [], [], hi, np.inf, 0)
    assert f1 is None
    ud = h1[-1:]
    h2, _, f2, _ = solver.explicit_dynamic_solver_v5(m["K"], m["C"], m["M"], t, [], [], fi, ud, hi, np.inf, 0)
    assert np.abs(h2 - h1).max() <= 1e-12 * np.abs(h1).max()
    assert np.abs(f2[0] - s).max() <= 1e-9 * np.abs(s).max()


def test_undamped_energy_is_bounded():
    m = modelgen.solid_plate(W=2e-3, H=1e-3, h=0.1e-3)
    nt = 400
    t, s = modelgen.pulse(nt, m["dt"])
    s[150:] = 0
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    _, fld, _, _ = solver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, fi, s, [], [], [],
                                                     25, 0, "KE", solver.VEL_CURRENT)
    mm = m["M"].diagonal()
    ke = 0.5 * (fld ** 2 * mm[:, None]).sum(0)
    late = ke[10:]
    assert late.max() < 4 * late[late > 0].mean()


def test_fluid_solid_reflection_normal_incidence():
    # Schmerr Eq. 6.122 at normal incidence (tests/fn_fluid_solid.m):
    # R = (Z_s - Z_f) / (Z_s + Z_f) for pressure.
    def fn_fluid_solid(theta, cf, rf, cl, cs, rs):
        tl = np.arcsin(np.sin(theta) * cl / cf)
        ts = np.arcsin(np.sin(theta) * cs / cf)
        d1 = np.cos(tl)
        d2 = (cl * rs) / (cf * rf) * np.cos(theta) * (np.cos(2 * ts) ** 2 + cs ** 2 * np.sin(2 * ts) * np.sin(2 * tl) / cl ** 2)
        return (d2 - d1) / (d1 + d2)
    R = fn_fluid_solid(0.0, 1500, 1000, 5940, 3200, 7900)
    Zs, Zf = 5940 * 7900, 1500 * 1000
    assert np.isclose(R, (Zs - Zf) / (Zs + Zf))


def test_bristolfe_entry_res_layout_and_wts_quirk():
    m = modelgen.solid_plate(W=1e-3, H=0.5e-3, h=0.1e-3)
    nt = 60
    t, s = modelgen.pulse(nt, m["dt"])
    mon = list(m["mon_nds"][:3]) + [m["mon_nds"][3]]
    steps = [dict(load=dict(time=t, frc_nds=[m["frc_nd"]], frc_dfs=[2], frcs=s, wts=[2.0]),
                  mon=dict(nds=mon, dfs=[2, 2, 2, 9 if False else 1])),
             dict(load=dict(time=t, frc_nds=[m["frc_nd"]], frc_dfs=[2], frcs=s, wts=[5.0]),
                  mon=dict(nds=mon, dfs=[2, 2, 2, 1]))]
    res, mats = entry.BristolFE_v2(m["mod"], m["matls"], steps, dict(dof_to_use=[1, 2]))
    assert res[0]["dsps"].shape == (4, nt)
    # steps{1}.load.wts is used for every step (fn_BristolFE_v2.m:79)
    assert np.allclose(res[0]["dsps"], res[1]["dsps"])


def test_history_rows_grow_to_last_valid_monitor():
    # res.dsps(valid, :) = ... sizes the array to the last valid row (fn_BristolFE_v2.m:127)
    valid = np.array([True, False, True, False])
    out = entry._grow_rows(valid, np.ones((2, 5)), 5)
    assert out.shape == (3, 5) and np.all(out[1] == 0)


def test_ti_start_and_zero_forcing():
    m = modelgen.solid_plate(W=1e-3, H=0.5e-3, h=0.1e-3)
    nt = 50
    t = np.arange(nt) * m["dt"]
    s = np.zeros(nt); s[20] = 1.0
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    h, _, _, _ = solver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, fi, s, [], [], fi,
                                                   np.inf, 0, "KE", solver.VEL_CURRENT)
    assert np.all(h[:, :20] == 0) and h[0, 20] != 0
    h0, _, _, _ = solver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, fi, 0 * s, [], [], fi,
                                                    np.inf, 0, "KE", solver.VEL_CURRENT)
    assert np.all(h0 == 0)


def test_unknown_solver_mode_fails_like_reference():
    m = modelgen.solid_plate(W=0.5e-3, H=0.5e-3, h=0.1e-3)
    t = np.arange(10) * m["dt"]
    with pytest.raises(solver.SolverError):
        solver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, [1], np.ones(10), [], [], [1],
                                          np.inf, 0, "KE", "vel at current time step")


def _strip_speed(mat, dof, c_nominal, W=20e-3, H=0.4e-3, h=0.05e-3, f=2e6):
    """Speed of a plane pulse in a strip that carries one DOF: uniform force
    on the left edge, pulse delay between node lines at x = 3 and 6 mm from
    the cross-correlation peak (parabolic sub-sample fit). The window ends
    before the reflection from the far end (x = W) reaches the lines."""
    from oracle import assembly, mesh, signals
    mod = mesh.rectangular_structured_mesh(np.array([[0, 0], [W, 0], [W, H], [0, H]]), h)
    mod["el_typ_i"] = [mat["el_typ"]] * len(mod["el_mat_i"])
    K, C, M, gl = assembly.build_global_matrices_v5(mod["nds"], mod["els"], mod["el_mat_i"], mod["el_abs_i"],
                                                    mod["el_typ_i"], [mat], dict(dof_to_use=[dof]))
    x = mod["nds"][:, 0]
    d = 0 if gl.shape[1] == 1 else dof - 1
    left = np.nonzero(np.isclose(x, 0))[0]
    lines = [np.nonzero(np.isclose(x, xx))[0] for xx in (3e-3, 6e-3)]
    rho = mat["rho"]
    D = np.atleast_2d(mat["D"])
    dt = 0.5 * h / np.sqrt(D.max() / rho)
    n_t = int((6e-3 / c_nominal + 6.0 / f) / dt)          # travel to the far line + the pulse
    t = np.arange(n_t) * dt
    sig = signals.gaussian_pulse(t, f, 5)
    fi = gl[left, d]
    hi = np.concatenate([gl[ln, d] for ln in lines])
    U = solver.explicit_dynamic_solver_v6(K, C, M, t, fi, sig, [], [], hi, np.inf, 0, "KE", solver.VEL_CURRENT)[0]
    a = U[: lines[0].size].mean(axis=0)
    b = U[lines[0].size:].mean(axis=0)
    xc = np.correlate(b, a, mode="full")
    k = int(np.argmax(xc))
    y0, y1, y2 = xc[k - 1], xc[k], xc[k + 1]
    lag = (k - (n_t - 1)) + 0.5 * (y0 - y2) / (y0 - 2 * y1 + y2)
    return 3e-3 / (lag * dt)


def test_wave_speeds_match_the_material_constants():
    """Plane longitudinal and shear waves in steel (strips carrying only DOF 1
    or only DOF 2) and sound in water (DOF 4) travel at sqrt(D/rho): c_L =
    sqrt(D11/rho), c_S = sqrt(D66/rho), c = sqrt(bulk/rho), within 0.5 %
    (linear triangles at 30-60 elements per wavelength, where the scheme's
    dispersion is below that)."""
    steel = dict(rho=8000.0, D=signals.isotropic_stiffness_matrix(210e9, 0.3), el_typ="CPE3")
    water = dict(rho=1000.0, D=1500.0 ** 2 * 1000.0, el_typ="AC2D3")
    Ds = np.asarray(steel["D"])
    c_l = np.sqrt(Ds[0, 0] / steel["rho"])
    c_s = np.sqrt(Ds[-1, -1] / steel["rho"])
    cl = _strip_speed(steel, 1, c_l)
    cs = _strip_speed(steel, 2, c_s)
    cw = _strip_speed(water, 4, 1500.0, f=1e6)             # 30 elements per wavelength
    assert abs(cl / c_l - 1) <= 5e-3, cl
    assert abs(cs / c_s - 1) <= 5e-3, cs
    assert abs(cw / 1500.0 - 1) <= 5e-3, cw
