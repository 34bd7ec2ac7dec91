"""3D 8-node brick (no reference implementation: the reference names C3D8R
only for external solvers, examples/solid_example_3d.m:18). The oracle's
HEX8 restatement is pinned by FE identities; the product's structured
builder is checked against it; the GPU march against the oracle."""
import numpy as np
import pytest

import modelgen
from bfe_gb300 import model
from oracle import assembly, elements, mesh, signals
from oracle import solver as osolver

STEEL = modelgen.STEEL


def _brick(dx=1e-4, dy=1.2e-4, dz=0.9e-4):
    nds = np.array([[0, 0, 0], [dx, 0, 0], [dx, dy, 0], [0, dy, 0],
                    [0, 0, dz], [dx, 0, dz], [dx, dy, dz], [0, dy, dz]], float)
    K, C, M, ln, ld = elements.el_HEX8(nds, np.array([[1, 2, 3, 4, 5, 6, 7, 8]]), STEEL["D"], STEEL["rho"])
    return nds, K[0], M[0]


def test_hex8_symmetric_rigid_body_and_mass():
    nds, K, M = _brick()
    assert np.abs(K - K.T).max() <= 1e-12 * np.abs(K).max()
    modes = []
    for d in range(3):
        u = np.zeros((8, 3)); u[:, d] = 1; modes.append(u.ravel())
    for (a, b) in ((0, 1), (1, 2), (0, 2)):           # infinitesimal rotations
        u = np.zeros((8, 3)); u[:, a] = -nds[:, b]; u[:, b] = nds[:, a]; modes.append(u.ravel())
    for u in modes:
        assert np.abs(K @ u).max() <= 1e-9 * np.abs(K).max() * np.abs(u).max()
    ev = np.linalg.eigvalsh(K)
    assert (ev < 1e-9 * ev.max()).sum() == 6          # exactly six zero-energy modes
    assert np.isclose(M.sum() / 3, STEEL["rho"] * 1e-4 * 1.2e-4 * 0.9e-4, rtol=1e-12)


def test_hex8_patch_test_constant_strain():
    # a linear displacement field gives zero force at interior nodes of a patch
    o = mesh.cubic_structured_mesh_3d(np.array([[0, 0, 0], [0.3e-3, 0.3e-3, 0.3e-3]]), 0.1e-3)
    K, C, M, gl = assembly.build_global_matrices_v5(o["nds"], o["els"], np.ones(len(o["els"]), int),
                                                    np.zeros(len(o["els"])), ["HEX8"] * len(o["els"]),
                                                    [dict(STEEL, el_typ="HEX8")], {})
    A = np.array([[1.0, 0.3, -0.2], [0.1, -0.5, 0.4], [0.2, 0.7, 0.9]]) * 1e-3
    u = (o["nds"] @ A.T).ravel()
    f = K @ u
    x = o["nds"]
    interior = np.all((x > 1e-9) & (x < 0.3e-3 - 1e-9), axis=1)
    fi = f.reshape(-1, 3)[interior]
    assert np.abs(fi).max() <= 1e-8 * np.abs(f).max()


def test_brick_grid_builder_matches_oracle():
    m = model.steel_block_3d(Lx=1.2e-3, Ly=1.0e-3, Lz=0.8e-3, h=0.1e-3, abs_wavelengths=0.05)
    o = mesh.cubic_structured_mesh_3d(np.array([[0, 0, 0], [1.2e-3, 1.0e-3, 0.8e-3]]), 0.1e-3)
    assert np.array_equal(o["els"], m["els"])
    K, C, M, gl = assembly.build_global_matrices_v5(o["nds"], o["els"], np.ones(len(o["els"]), int),
                                                    m["el_abs"], ["HEX8"] * len(o["els"]),
                                                    [dict(STEEL, el_typ="HEX8")], {})
    rel = lambda A, B: (abs(A - B).max() if abs(A - B).nnz else 0.0) / abs(B).max()
    assert np.array_equal(gl, m["gl"])
    assert rel(m["K"], K) < 1e-13 and rel(m["M"], M) < 1e-13 and rel(m["C"], C) < 1e-13


@pytest.fixture(scope="module")
def block():
    return model.steel_block_3d(Lx=1.6e-3, Ly=1.4e-3, Lz=1.0e-3, h=0.1e-3, abs_wavelengths=0.25,
                                n_mon=16)


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


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [("double", 1e-10), ("single", 1e-4)])
def test_hex3d_march_matches_oracle(bfe, block, prec, tol):
    m = block
    nt = 300
    t, s = modelgen.pulse(nt, m["dt"])
    fi = model.global_indices(m["gl"], m["src_nodes"][0], 3)
    hi = model.global_indices(m["gl"], m["mon_nodes"], 3)
    h0, _, _, _ = osolver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, fi, s, [], [], hi,
                                                     np.inf, 0, "KE", osolver.VEL_CURRENT)
    h1, _, _, _ = bfe.fn_explicit_dynamic_solver_gb300(m["K"], m["C"], m["M"], t, fi, s, [], [], hi,
                                                       np.inf, 1, "KE", osolver.VEL_CURRENT, prec,
                                                       gl_lookup=m["gl"])
    assert np.abs(h1 - h0).max() <= tol * np.abs(h0).max()


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [0, 9, 13, 14, 20])
def test_hex3d_batched_fp32_matches_oracle(bfe, block, variant, monkeypatch):
    m = block
    nt = 200
    t, s = modelgen.pulse(nt, m["dt"])
    top = m["mon_nodes"]
    srcs = [model.global_indices(m["gl"], [top[r % top.size]], 3) for r in range(64)]
    hi = model.global_indices(m["gl"], m["mon_nodes"], 3)
    monkeypatch.setenv("BFE_VARIANT", str(variant))
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], osolver.VEL_CURRENT, "single", m["gl"]) as plan:
        hb = plan.run_batched(t, srcs, s, hi)
        st = plan.stats()
    assert st["n_groups"] == 1 and st["variant"] == variant
    for r in (0, 5):
        h0, _, _, _ = osolver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, srcs[r], s, [], [], hi,
                                                         np.inf, 0, "KE", osolver.VEL_CURRENT)
        assert np.abs(hb[:, :, r] - h0).max() <= 1e-4 * np.abs(h0).max()
