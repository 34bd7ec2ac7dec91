"""The allocation-free entry point bfe_run_f64_noalloc.

Some callers cannot call cudaMalloc (their device memory belongs to a
framework allocator or a fixed pool, or they must avoid the synchronisation
that allocating implies mid-pipeline). This test plays such a caller: it
keeps operator, signals and history in device memory it already owns, calls
the allocation-free march through the C ABI twice in a row, and checks both
results against the existing entry point (bfe_run through a plan) within the
FP64 tolerance of the other tests. The file name sorts last so that a
stop-at-first-failure run has run every other test first.
"""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp

import modelgen
from oracle import solver as osolver

pytestmark = pytest.mark.gpu

TOL64 = 1e-10


@pytest.fixture(scope="module")
def lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from bfe_gb300 import _lib, build
    build.build()
    return _lib, _lib.load()


def _operators(m):
    """Reference operators for a diagonal P: B = P^-1 (2I - dt^2 M^-1 K),
    d = P^-1 (-1 + gamma), a = P^-1 dt^2 / m (fn_explicit_dynamic_solver_v6.m:135-138)."""
    K, C, M, dt = m["K"], m["C"], m["M"], m["dt"]
    mm = np.asarray(M.sum(0)).ravel()
    gam = dt / 2 * C.diagonal() / mm
    p = 1.0 / (1.0 + gam)
    n = K.shape[0]
    B = (sp.diags(p) @ (2 * sp.identity(n) - sp.diags(dt ** 2 / mm) @ K)).tocsr()
    B.sort_indices()
    return B, p * (-1.0 + gam), p * dt ** 2 / mm


def test_noalloc_matches_plan_run_twice(lib):
    import torch
    L, so = lib
    import bfe_gb300
    m = modelgen.solid_plate(W=3e-3, H=1.5e-3, h=0.1e-3, abs_thick=0.3e-3)
    assert abs(m["C"] - sp.diags(m["C"].diagonal())).sum() == 0    # diagonal P
    nt = 500
    t, s = modelgen.pulse(nt, m["dt"])
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    hi = modelgen.gi_of(m["gl"], m["mon_nds"], 2)
    with bfe_gb300.Plan(m["K"], m["C"], m["M"], m["dt"], osolver.VEL_CURRENT, "double") as plan:
        h_ref, _, _ = plan.run(t, fi, s, hi)

    B, dvec, acoef = _operators(m)
    n = B.shape[0]
    dev = torch.device("cuda")
    d_rp = torch.tensor(B.indptr.astype(np.int32), device=dev)
    d_ci = torch.tensor(B.indices.astype(np.int32), device=dev)
    d_bv = torch.tensor(B.data, dtype=torch.float64, device=dev)
    d_dv = torch.tensor(dvec, dtype=torch.float64, device=dev)
    d_frow = torch.tensor((fi - 1).astype(np.int32), device=dev)
    d_fcoef = torch.tensor(acoef[fi - 1], dtype=torch.float64, device=dev)
    d_sig = torch.tensor(s.reshape(nt, 1), dtype=torch.float64, device=dev)
    d_hrow = torch.tensor((hi - 1).astype(np.int32), device=dev)
    ti0 = int(np.nonzero(s)[0].min())
    stream = torch.cuda.current_stream().cuda_stream

    def call(d_hist):
        return so.bfe_run_f64_noalloc(
            n, ctypes.c_void_p(d_rp.data_ptr()), ctypes.c_void_p(d_ci.data_ptr()),
            ctypes.c_void_p(d_bv.data_ptr()), ctypes.c_void_p(d_dv.data_ptr()),
            nt, ti0, fi.size, ctypes.c_void_p(d_frow.data_ptr()),
            ctypes.c_void_p(d_fcoef.data_ptr()), ctypes.c_void_p(d_sig.data_ptr()),
            hi.size, ctypes.c_void_p(d_hrow.data_ptr()), ctypes.c_void_p(d_hist.data_ptr()),
            ctypes.c_void_p(stream))

    scale = np.abs(h_ref).max()
    for _ in range(2):                                   # the array keeps the last call's state
        d_hist = torch.zeros((nt, hi.size), dtype=torch.float64, device=dev)   # q x n_t column-major
        assert call(d_hist) == L.BFE_OK, so.bfe_last_error()
        h = d_hist.cpu().numpy().T
        assert np.abs(h - h_ref).max() <= TOL64 * scale


def test_noalloc_rejects_oversized_models(lib):
    L, so = lib
    st = so.bfe_run_f64_noalloc((1 << 20) + 1, None, None, None, None, 10, 0, 0, None, None, None,
                                0, None, None, None)
    assert st == L.BFE_ERR_ARG
    assert b"1048576" in so.bfe_last_error()
