"""The product's synthetic model generators (bfe_gb300.model) against the
oracle's restatements of the reference's mesh, material, absorbing-layer,
interface and assembly functions (fn_rectangular_structured_mesh,
fn_set_els_inside_bdry_to_mat, fn_add_absorbing_layer,
fn_add_fluid_solid_interface_els, fn_build_global_matrices_v5): given the
same void polygon, both build the same K, C and M (small models, CPU)."""
import numpy as np

from bfe_gb300 import model
from oracle import assembly, mesh, signals

STEEL = dict(rho=8000.0, D=signals.isotropic_stiffness_matrix(210e9, 0.3), el_typ="CPE3")
WATER = dict(rho=1000.0, D=1500.0 ** 2 * 1000.0, el_typ="AC2D3")


def _same(a, b):
    assert a.shape == b.shape
    return abs(a - b).max() <= 1e-14 * abs(b).max()


def test_steel_subdomain_matches_the_reference_pipeline():
    side, h, fc, seed = 3e-3, 0.1e-3, 5e6, 5
    m = model.steel_subdomain(side, h=h, fc=fc, seed=seed, n_src=4, n_mon=4)
    blob = model.smooth_blob(min(1.5e-3, side / 8), 8, 0.2, np.random.default_rng(seed)) + side / 2
    mod = mesh.rectangular_structured_mesh(np.array([[0, 0], [side, 0], [side, side], [0, side]]), h)
    mod = mesh.remove_elements_in_region(mod, blob)
    th = min(3.0 * np.sqrt(STEEL["D"][0, 0] / STEEL["rho"]) / fc, side / 4)
    mod = mesh.add_absorbing_layer(mod, np.array([[th, th], [side - th, th], [side - th, side - th],
                                                  [th, side - th]]), th)
    mod["el_typ_i"] = ["CPE3"] * len(mod["el_mat_i"])
    K, C, M, gl = assembly.build_global_matrices_v5(mod["nds"], mod["els"], mod["el_mat_i"], mod["el_abs_i"],
                                                    mod["el_typ_i"], [STEEL], dict(dof_to_use=[1, 2],
                                                                                   damping_power_law=2))
    assert _same(K, m["K"]) and _same(C, m["C"]) and _same(M, m["M"])
    assert np.array_equal(np.asarray(gl), np.asarray(m["gl"]))


def test_coupled_model_matches_the_reference_pipeline():
    W, Hw, Hs, h, fc = 6e-3, 2e-3, 1.5e-3, 0.1e-3, 20e6
    blob = model.smooth_blob(0.4e-3, 8, 0.2, np.random.default_rng(3)) + np.array([W / 2, Hs / 2])
    m = model.coupled_water_steel(W=W, H_water=Hw, H_steel=Hs, h=h, fc=fc, blob_polygon_pts=blob,
                                  array_elements=4, array_pitch=0.6e-3)
    Ht = Hw + Hs
    matls = [STEEL, WATER]
    mod = mesh.rectangular_structured_mesh(np.array([[0, 0], [W, 0], [W, Ht], [0, Ht]]), h)
    mod = mesh.set_els_inside_bdry_to_mat(mod, np.array([[-1, Hs], [W + 1, Hs], [W + 1, Ht + 1], [-1, Ht + 1]]), 2)
    mod = mesh.remove_elements_in_region(mod, blob)
    mod["el_typ_i"] = [matls[k - 1]["el_typ"] for k in mod["el_mat_i"]]
    th = 3.0 * np.sqrt(STEEL["D"][0, 0] / STEEL["rho"]) / fc
    mod = mesh.add_absorbing_layer(mod, np.array([[th, th], [W - th, th], [W - th, Ht + 1.0], [th, Ht + 1.0]]), th)
    mod = mesh.add_fluid_solid_interface_els(mod, matls)
    K, C, M, gl = assembly.build_global_matrices_v5(mod["nds"], mod["els"], mod["el_mat_i"], mod["el_abs_i"],
                                                    mod["el_typ_i"], matls,
                                                    dict(dof_to_use=[1, 2, 4], damping_power_law=2))
    assert _same(K, m["K"]) and _same(C, m["C"]) and _same(M, m["M"])
    assert np.array_equal(np.asarray(gl), np.asarray(m["gl"]))


def test_plate_matches_the_reference_pipeline_and_time_step():
    """The C0 plate (DOFs 1-2 and the default 1-3): same K, C, M and
    gl_lookup, and the same element-eigenvalue time step."""
    W, H, h = 3e-3, 1.5e-3, 0.1e-3
    for dofs in ((1, 2), (1, 2, 3)):
        m = model.steel_plate(W=W, H=H, h=h, n_mon=4, dof_to_use=dofs)
        mod = mesh.rectangular_structured_mesh(np.array([[0, 0], [W, 0], [W, H], [0, H]]), h)
        mod["el_typ_i"] = ["CPE3"] * len(mod["el_mat_i"])
        K, C, M, gl = assembly.build_global_matrices_v5(mod["nds"], mod["els"], mod["el_mat_i"], mod["el_abs_i"],
                                                        mod["el_typ_i"], [STEEL], dict(dof_to_use=list(dofs)))
        assert _same(K, m["K"]) and _same(M, m["M"]) and abs(C).sum() == abs(m["C"]).sum() == 0
        assert np.array_equal(np.asarray(gl), np.asarray(m["gl"]))
        dt = signals.element_eigen_time_step(mod["nds"], mod["els"], STEEL["D"], STEEL["rho"])
        assert abs(dt - m["dt"]) <= 1e-12 * dt
