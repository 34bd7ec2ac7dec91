"""Small seeded test models built with the oracle's restated generators.

Test infrastructure only (imports the oracle).
"""
import numpy as np

from oracle import assembly, mesh, signals

STEEL = dict(rho=8000.0, D=signals.isotropic_stiffness_matrix(210e9, 0.3), el_typ="CPE3")
WATER = dict(rho=1000.0, D=1500.0 ** 2 * 1000.0, el_typ="AC2D3")


def solid_plate(W=4e-3, H=2e-3, h=0.1e-3, dof_to_use=(1, 2), abs_thick=0.0, n_mon=16):
    """Steel plate (fn_rectangular_structured_mesh), vertical point force at the
    top-surface centre node, monitors along the top surface."""
    matls = [dict(STEEL)]
    bdry = np.array([[0, 0], [W, 0], [W, H], [0, H]])
    mod = mesh.rectangular_structured_mesh(bdry, h)
    typ = ["CPE3"] * mod["els"].shape[0]
    opts = dict(dof_to_use=list(dof_to_use))
    if abs_thick > 0:
        inner = np.array([[abs_thick, abs_thick], [W - abs_thick, abs_thick],
                          [W - abs_thick, H + 1e-9], [abs_thick, H + 1e-9]])
        mod = mesh.add_absorbing_layer(mod, inner, abs_thick)
    K, C, M, gl = assembly.build_global_matrices_v5(mod["nds"], mod["els"], mod["el_mat_i"],
                                                    mod["el_abs_i"], typ, matls, opts)
    dt = signals.element_eigen_time_step(mod["nds"], mod["els"], STEEL["D"], STEEL["rho"])
    top = np.nonzero(np.isclose(mod["nds"][:, 1], H))[0]
    ctr = top[np.argmin(np.abs(mod["nds"][top, 0] - W / 2))]
    mon_nds = top[np.linspace(0, top.size - 1, n_mon).astype(int)]
    return dict(mod=mod, matls=matls, typ=typ, K=K, C=C, M=M, gl=gl, dt=dt,
                frc_nd=ctr + 1, mon_nds=mon_nds + 1)


def coupled_model(W=3e-3, Hw=1.5e-3, Hs=1.5e-3, h=0.1e-3, abs_thick=0.6e-3,
                  dof_to_use=(1, 2, 4), blob=False, seed=0):
    """Water over steel (fn_set_els_inside_bdry_to_mat) with ASI2D2 interface
    elements (fn_add_fluid_solid_interface_els) and absorbing layers on the
    left, right and bottom (fn_add_absorbing_layer)."""
    matls = [dict(STEEL), dict(WATER)]
    H = Hw + Hs
    bdry = np.array([[0, 0], [W, 0], [W, H], [0, H]])
    mod = mesh.rectangular_structured_mesh(bdry, h)
    mod["el_mat_i"][:] = 1
    water = np.array([[-1, Hs], [W + 1, Hs], [W + 1, H + 1], [-1, H + 1]])
    mod = mesh.set_els_inside_bdry_to_mat(mod, water, 2)
    if blob:
        rng = np.random.default_rng(seed)
        pts = mesh.create_smooth_random_blob(0.5, 4, 64, rng) * (Hs / 5) + np.array([W / 2, Hs / 2])
        mod = mesh.remove_elements_in_region(mod, pts)
    mod["el_typ_i"] = [matls[m - 1]["el_typ"] for m in mod["el_mat_i"]]
    if abs_thick > 0:
        inner = np.array([[abs_thick, abs_thick], [W - abs_thick, abs_thick],
                          [W - abs_thick, H + 1], [abs_thick, H + 1]])
        mod = mesh.add_absorbing_layer(mod, inner, abs_thick)
    else:
        mod["el_abs_i"] = np.zeros(mod["els"].shape[0])
    mod = mesh.add_fluid_solid_interface_els(mod, matls)
    opts = dict(dof_to_use=list(dof_to_use), damping_power_law=2)
    K, C, M, gl = assembly.build_global_matrices_v5(mod["nds"], mod["els"], mod["el_mat_i"],
                                                    mod["el_abs_i"], mod["el_typ_i"], matls, opts)
    solid = np.array([t == "CPE3" for t in mod["el_typ_i"]])
    dt = signals.element_eigen_time_step(mod["nds"], mod["els"][solid, :3], STEEL["D"], STEEL["rho"])
    top = np.nonzero(np.isclose(mod["nds"][:, 1], H))[0]
    src = top[np.argmin(np.abs(mod["nds"][top, 0] - W / 2))]
    iface = np.nonzero(np.isclose(mod["nds"][:, 1], Hs))[0]
    mon = np.concatenate([top[:: max(1, top.size // 8)], iface[:: max(1, iface.size // 8)]])
    return dict(mod=mod, matls=matls, K=K, C=C, M=M, gl=gl, dt=dt, frc_nd=src + 1,
                mon_nds=mon + 1)


def pulse(nt, dt, f=5e6, cycles=5):
    t = np.arange(nt) * dt
    return t, signals.gaussian_pulse(t, f, cycles)


def gi_of(gl, nds, dof):
    """1-based global indices of (node, dof) pairs (fn_nds_and_dfs_to_gi)."""
    g = gl[np.asarray(nds) - 1, dof - 1]
    return g[g > 0]
