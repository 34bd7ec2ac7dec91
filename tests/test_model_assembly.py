"""Product model builder (bfe_gb300.model) against the oracle: identical mesh
numbering, identical interface elements, bit-exact DOF numbering (gl_lookup)
and K, C, M equal to FP64 rounding."""
import numpy as np
import pytest

import modelgen
from bfe_gb300 import model
from oracle import assembly, mesh


def _rel(A, B):
    d = abs(A - B)
    return (d.max() if d.nnz else 0.0) / max(abs(B).max(), 1e-300)


def test_rect_mesh_matches_reference_order():
    W, H, h = 1.3e-3, 0.7e-3, 0.1e-3
    o = mesh.rectangular_structured_mesh(np.array([[0, 0], [W, 0], [W, H], [0, H]]), h)
    nds, els = model.rect_mesh(0.0, W, 0.0, H, h)
    assert np.array_equal(els, o["els"])
    assert np.allclose(nds, o["nds"], rtol=0, atol=1e-15)


def test_plate_assembly_with_absorbers_matches_oracle():
    m = modelgen.solid_plate(W=2e-3, H=1e-3, h=0.1e-3, abs_thick=0.3e-3)
    mod = m["mod"]
    D = model.isotropic_stiffness(210e9, 0.3)
    typ = np.zeros(mod["els"].shape[0], np.int64)
    K, C, M, gl = model.assemble(mod["nds"], mod["els"], mod["el_mat_i"], mod["el_abs_i"], typ,
                                 [dict(D=D, rho=8000.0)], [1, 2])
    assert np.array_equal(gl, m["gl"])
    assert _rel(K, m["K"]) < 1e-13 and _rel(M, m["M"]) < 1e-13 and _rel(C, m["C"]) < 1e-13


@pytest.mark.parametrize("dofs", [(1, 2, 4), ()])
def test_coupled_assembly_matches_oracle(dofs):
    m = modelgen.coupled_model(W=2e-3, Hw=1e-3, Hs=1e-3, h=0.1e-3, abs_thick=0.4e-3,
                               dof_to_use=dofs if dofs else [], blob=True)
    mod = m["mod"]
    names = mod["el_typ_i"]
    typ = np.array([model.TYPE_CODES[t] for t in names])
    matls = [dict(D=model.isotropic_stiffness(210e9, 0.3), rho=8000.0),
             dict(D=1500.0 ** 2 * 1000.0, rho=1000.0)]
    K, C, M, gl = model.assemble(mod["nds"], mod["els"], mod["el_mat_i"], mod["el_abs_i"], typ,
                                 matls, list(dofs) if dofs else None, damping_power_law=2)
    assert np.array_equal(gl, m["gl"])
    assert _rel(K, m["K"]) < 1e-13 and _rel(M, m["M"]) < 1e-13 and _rel(C, m["C"]) < 1e-13


def test_interface_elements_match_oracle():
    m = modelgen.coupled_model(W=2e-3, Hw=1e-3, Hs=1e-3, h=0.1e-3, abs_thick=0.0, blob=True)
    mod = m["mod"]
    typ = np.array([model.TYPE_CODES[t] for t in mod["el_typ_i"]])
    tri = typ != model.TYPE_CODES["ASI2D2"]
    ed = model.fluid_solid_interfaces(mod["nds"], mod["els"][tri], typ[tri])
    ref = mod["els"][~tri][:, :2]
    assert np.array_equal(ed, ref)


def test_absorbing_index_matches_oracle():
    nds, els = model.rect_mesh(0.0, 2e-3, 0.0, 1e-3, 0.1e-3)
    inner = np.array([[0.3e-3, 0.3e-3], [1.7e-3, 0.3e-3], [1.7e-3, 2.0], [0.3e-3, 2.0]])
    o = mesh.add_absorbing_layer(dict(nds=nds, els=els), inner, 0.3e-3)
    ctr = model.centroids(nds, els)
    a = np.clip(model.distance_to_polygon(ctr, inner) / 0.3e-3, 0, 1)
    a[model.points_in_polygon(ctr, inner)] = 0
    assert np.allclose(a, o["el_abs_i"], rtol=0, atol=1e-12)


def test_toneburst_matches_oracle():
    from oracle import signals
    t = np.arange(700) * 9.7e-9
    assert np.allclose(model.toneburst(t, 5e6, 5), signals.gaussian_pulse(t, 5e6, 5), rtol=0, atol=1e-15)


def test_element_stable_dt_matches_oracle():
    from oracle import signals
    nds, els = model.rect_mesh(0.0, 1e-3, 0.0, 1e-3, 0.1e-3)
    D = model.isotropic_stiffness(210e9, 0.3)
    assert np.isclose(model.element_stable_dt(nds, els, D, 8000.0),
                      signals.element_eigen_time_step(nds, els, D, 8000.0), rtol=1e-12)
