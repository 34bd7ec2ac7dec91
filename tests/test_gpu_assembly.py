"""GPU global assembly (bfe_assemble_2d) against the oracle's restatement of
fn_build_global_matrices_v5: identical gl_lookup and sparsity, values within
1e-13 of the largest entry (FP64, summation order may differ); a plan built
from the device matrices marches like the oracle."""
import numpy as np
import pytest

import modelgen
from oracle import assembly as oassembly
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


def _compare(got, ref):
    K, C, M, gl = got
    Ko, Co, Mo, glo = ref
    assert np.array_equal(gl, glo)
    for a, b in ((K, Ko), (C, Co), (M, Mo)):
        a, b = a.tocsr(), b.tocsr()
        a.sort_indices()
        b.sort_indices()
        assert a.shape == b.shape
        assert np.array_equal(a.indptr, b.indptr) and np.array_equal(a.indices, b.indices)
        scale = max(abs(b).max(), 1e-300)
        assert np.abs(a.data - b.data).max() <= 1e-13 * scale


def _oracle(mod, matls, opts):
    return oassembly.build_global_matrices_v5(mod["nds"], mod["els"], mod["el_mat_i"], mod["el_abs_i"],
                                              mod["el_typ_i"], matls, opts)


def _gpu(bfe, mod, matls, dof_to_use=None, pw=3):
    return bfe.assemble_gpu(mod["nds"], mod["els"], mod["el_mat_i"], mod["el_abs_i"], mod["el_typ_i"],
                            matls, dof_to_use=dof_to_use, damping_power_law=pw)


@pytest.mark.parametrize("dofs", [(1, 2), None])
def test_plate_with_absorbers(bfe, dofs):
    m = modelgen.solid_plate(W=3e-3, H=2e-3, h=0.1e-3, dof_to_use=dofs or (1, 2, 3), abs_thick=0.5e-3)
    mod = dict(m["mod"], el_typ_i=m["typ"])
    opts = {} if dofs is None else dict(dof_to_use=list(dofs))
    _compare(_gpu(bfe, mod, m["matls"], dofs), _oracle(mod, m["matls"], opts))


@pytest.mark.parametrize("dofs", [(1, 2, 4), None])
def test_coupled_model_with_interface_and_void(bfe, dofs):
    m = modelgen.coupled_model(W=3e-3, Hw=1.5e-3, Hs=1.5e-3, h=0.1e-3, abs_thick=0.6e-3, blob=True)
    opts = dict(damping_power_law=2)
    if dofs:
        opts["dof_to_use"] = list(dofs)
    _compare(_gpu(bfe, m["mod"], m["matls"], dofs, pw=2), _oracle(m["mod"], m["matls"], opts))


def test_plan_from_device_matrices_marches_like_the_oracle(bfe):
    m = modelgen.coupled_model(W=3e-3, Hw=1.5e-3, Hs=1.5e-3, h=0.1e-3, abs_thick=0.6e-3, blob=True)
    mod = m["mod"]
    t, s = modelgen.pulse(500, m["dt"])
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 4)
    hi = modelgen.gi_of(m["gl"], m["mon_nds"], 4)
    h0, _, _, _ = osolver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, fi, s, [], [], hi, np.inf, 0,
                                                     "KE", osolver.VEL_CURRENT)
    with bfe.DeviceMatrices(mod["nds"], mod["els"], mod["el_mat_i"], mod["el_abs_i"], mod["el_typ_i"],
                            m["matls"], dof_to_use=(1, 2, 4), damping_power_law=2) as dm:
        assert np.array_equal(dm.gl_lookup(), m["gl"])
        for prec, tol in (("double", 1e-10), ("single", 1e-4)):
            with dm.plan(m["dt"], osolver.VEL_CURRENT, prec) as plan:
                h1, _, _ = plan.run(t, fi, s, hi)
            assert np.abs(h1 - h0).max() <= tol * np.abs(h0).max()
