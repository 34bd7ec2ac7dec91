"""The allocation-free entry point bfe_run_f64_noalloc.

Some callers cannot call cudaMalloc (their device memory belongs to a
framework allocator or a fixed pool, or they must avoid the synchronisation
that allocating implies mid-pipeline). These tests play such a caller: they
keep operator, signals and history in device memory they already own, call
the allocation-free march through the C ABI twice in a row, and check both
results against the existing entry point (bfe_run through a plan) and the
FP64 oracle within the FP64 tolerance of the other tests. Further cases: a
march from the first sample, no forcing and no monitors, history samples
before the first forced sample left as the caller filled them, repeated
forced rows (which add up), and the host-side argument errors (these need no
GPU). The file name sorts last so that a stop-at-first-failure run has run
every other test first.
"""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp

import modelgen
from oracle import solver as osolver

TOL64 = 1e-10


def _load():
    from bfe_gb300 import _lib, build
    build.build()
    return _lib, _lib.load()


@pytest.fixture(scope="module")
def lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return _load()


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


class _Caller:
    """A caller that owns its device buffers and calls the entry point."""

    def __init__(self, so, m, nt, frc_rows0, frc_weights, sig_cols, hist_rows0):
        import torch
        self.so = so
        B, dvec, acoef = _operators(m)
        self.n = B.shape[0]
        self.nt = nt
        dev = torch.device("cuda")
        self.keep = []

        def dt_(a, dtype):
            t = torch.tensor(a, dtype=dtype, device=dev)
            self.keep.append(t)
            return t
        self.d_rp = dt_(B.indptr.astype(np.int32), torch.int32)
        self.d_ci = dt_(B.indices.astype(np.int32), torch.int32)
        self.d_bv = dt_(B.data, torch.float64)
        self.d_dv = dt_(dvec, torch.float64)
        frc_rows0 = np.asarray(frc_rows0, np.int64)
        self.n_frc = frc_rows0.size
        self.d_frow = dt_(frc_rows0.astype(np.int32), torch.int32)
        self.d_fcoef = dt_(acoef[frc_rows0] * np.asarray(frc_weights, float), torch.float64)
        self.d_sig = dt_(np.ascontiguousarray(np.asarray(sig_cols, float).reshape(nt, self.n_frc)),
                         torch.float64)
        hist_rows0 = np.asarray(hist_rows0, np.int64)
        self.q = hist_rows0.size
        self.d_hrow = dt_(hist_rows0.astype(np.int32), torch.int32)
        self.stream = torch.cuda.current_stream().cuda_stream

    def __call__(self, d_hist, ti0):
        vp = ctypes.c_void_p
        return self.so.bfe_run_f64_noalloc(
            self.n, vp(self.d_rp.data_ptr()), vp(self.d_ci.data_ptr()), vp(self.d_bv.data_ptr()),
            vp(self.d_dv.data_ptr()), self.nt, ti0, self.n_frc,
            vp(self.d_frow.data_ptr() if self.n_frc else 0), vp(self.d_fcoef.data_ptr() if self.n_frc else 0),
            vp(self.d_sig.data_ptr() if self.n_frc else 0), self.q,
            vp(self.d_hrow.data_ptr() if self.q else 0), vp(d_hist.data_ptr() if d_hist is not None else 0),
            vp(self.stream))


def _plate():
    m = modelgen.solid_plate(W=3e-3, H=1.5e-3, h=0.1e-3, abs_thick=0.3e-3)
    assert abs(m["C"] - sp.diags(m["C"].diagonal())).sum() == 0    # diagonal P
    return m


@pytest.mark.gpu
def test_noalloc_matches_plan_run_and_oracle_twice(lib):
    import torch
    import bfe_gb300
    L, so = lib
    m = _plate()
    nt = 500
    t, s = modelgen.pulse(nt, m["dt"])
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    hi = modelgen.gi_of(m["gl"], m["mon_nds"], 2)
    with bfe_gb300.Plan(m["K"], m["C"], m["M"], m["dt"], osolver.VEL_CURRENT, "double") as plan:
        h_ref, _, _ = plan.run(t, fi, s, hi)
    h_orc, _, _, _ = osolver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, fi, s, [], [], hi,
                                                        np.inf, 0, "KE", osolver.VEL_CURRENT)
    call = _Caller(so, m, nt, fi - 1, np.ones(fi.size), np.repeat(s[:, None], fi.size, 1), hi - 1)
    ti0 = int(np.nonzero(s)[0].min())
    scale = np.abs(h_ref).max()
    for _ in range(2):                                   # the array keeps the last call's state
        d_hist = torch.zeros((nt, hi.size), dtype=torch.float64, device="cuda")   # q x n_t column-major
        assert call(d_hist, ti0) == L.BFE_OK, so.bfe_last_error()
        h = d_hist.cpu().numpy().T
        assert np.abs(h - h_ref).max() <= TOL64 * scale
        assert np.abs(h - h_orc).max() <= TOL64 * np.abs(h_orc).max()


@pytest.mark.gpu
def test_noalloc_edge_cases(lib):
    import torch
    L, so = lib
    m = _plate()
    nt = 300
    t, s = modelgen.pulse(nt, m["dt"])
    s = np.concatenate([np.zeros(25), s[:-25]])        # the forcing starts at sample 25
    fi = modelgen.gi_of(m["gl"], [m["frc_nd"]], 2)
    hi = modelgen.gi_of(m["gl"], m["mon_nds"], 2)
    ti0 = int(np.nonzero(s)[0].min())
    assert ti0 == 25
    h_orc, _, _, _ = osolver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, fi, s, [], [], hi,
                                                        np.inf, 0, "KE", osolver.VEL_CURRENT)
    scale = np.abs(h_orc).max()
    call = _Caller(so, m, nt, fi - 1, np.ones(fi.size), s[:, None], hi - 1)
    # a march from the first sample equals the one from ti0: the state stays
    # zero while the forcing is zero
    d_hist = torch.zeros((nt, hi.size), dtype=torch.float64, device="cuda")
    assert call(d_hist, 0) == L.BFE_OK, so.bfe_last_error()
    assert np.abs(d_hist.cpu().numpy().T - h_orc).max() <= TOL64 * scale
    # samples before ti_start keep what the caller put there
    d_hist = torch.full((nt, hi.size), 7.25, dtype=torch.float64, device="cuda")
    assert call(d_hist, ti0) == L.BFE_OK, so.bfe_last_error()
    h = d_hist.cpu().numpy().T
    assert np.all(h[:, :ti0] == 7.25)
    assert np.abs(h[:, ti0:] - h_orc[:, ti0:]).max() <= TOL64 * scale
    # no forcing: the history stays zero; no monitors: nothing is written
    quiet = _Caller(so, m, nt, [], [], np.zeros((nt, 0)), hi - 1)
    d_hist = torch.full((nt, hi.size), 1.0, dtype=torch.float64, device="cuda")
    assert quiet(d_hist, 0) == L.BFE_OK, so.bfe_last_error()
    assert np.all(d_hist.cpu().numpy() == 0.0)
    blind = _Caller(so, m, nt, fi - 1, np.ones(fi.size), s[:, None], [])
    assert blind(None, ti0) == L.BFE_OK, so.bfe_last_error()
    # a forced row named twice adds its two entries: weights 0.25 and 0.75
    # on the same row equal one entry of weight 1
    twice = _Caller(so, m, nt, np.repeat(fi - 1, 2), np.tile([0.25, 0.75], fi.size),
                    np.repeat(s[:, None], 2 * fi.size, 1), hi - 1)
    d_hist = torch.zeros((nt, hi.size), dtype=torch.float64, device="cuda")
    assert twice(d_hist, ti0) == L.BFE_OK, so.bfe_last_error()
    assert np.abs(d_hist.cpu().numpy().T - h_orc).max() <= TOL64 * scale


def test_noalloc_rejects_bad_arguments_on_the_host():
    """Argument errors return before any device work (no GPU needed)."""
    L, so = _load()
    vp = ctypes.c_void_p
    one = vp(16)                   # never dereferenced: every case fails its checks first
    ops = (one, one, one, one)
    st = so.bfe_run_f64_noalloc((1 << 20) + 1, *ops, 10, 0, 0, None, None, None, 0, None, None, None)
    assert st == L.BFE_ERR_ARG and b"1048576" in so.bfe_last_error()
    assert so.bfe_run_f64_noalloc(0, *ops, 10, 0, 0, None, None, None, 0, None, None, None) == L.BFE_ERR_ARG
    assert so.bfe_run_f64_noalloc(8, *ops, 0, 0, 0, None, None, None, 0, None, None, None) == L.BFE_ERR_ARG
    assert so.bfe_run_f64_noalloc(8, *ops, 10, -1, 0, None, None, None, 0, None, None, None) == L.BFE_ERR_ARG
    # counts beyond int32
    st = so.bfe_run_f64_noalloc(8, *ops, 10, 0, 1 << 31, one, one, one, 0, None, None, None)
    assert st == L.BFE_ERR_ARG and b"2147483647" in so.bfe_last_error()
    st = so.bfe_run_f64_noalloc(8, *ops, 10, 0, 0, None, None, None, 1 << 31, one, one, None)
    assert st == L.BFE_ERR_ARG
    # NULL operator, forcing and history arrays
    for k in range(4):
        args = list(ops)
        args[k] = None
        assert so.bfe_run_f64_noalloc(8, *args, 10, 0, 0, None, None, None, 0, None, None,
                                      None) == L.BFE_ERR_ARG
    for miss in range(3):
        f = [one, one, one]
        f[miss] = None
        assert so.bfe_run_f64_noalloc(8, *ops, 10, 0, 1, *f, 0, None, None, None) == L.BFE_ERR_ARG
    for miss in range(2):
        h = [one, one]
        h[miss] = None
        assert so.bfe_run_f64_noalloc(8, *ops, 10, 0, 0, None, None, None, 2, *h, None) == L.BFE_ERR_ARG
