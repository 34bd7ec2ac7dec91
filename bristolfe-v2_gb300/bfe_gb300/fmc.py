"""Sub-domain and FMC post-processing on the GPU, mirroring the reference's
fn_convolve (code/internal/fn_convolve.m), fn_parse_to_fmc
(subdoms/fn_run_main_model.m:239-256) and fn_convert_disps_to_forces_v2
(code/fn_convert_disps_to_forces_v2.m) over the native kernels.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, ptr
from .solver import VEL_CURRENT, VEL_LAST_HALF, SolverError, _csr_view


def fn_convolve_gb300(f, g, dim=1):
    """fn_convolve(f, g, dim) (code/internal/fn_convolve.m:22-33) on the GPU
    for dim = 1: each column of f with g, as the 2 size(f, 1)-point FFT
    convolution truncated to size(f) (a direct sum here, wrap-around
    included). A vector f is one signal. Returns an array shaped like f."""
    if dim != 1:
        raise SolverError("only dim = 1 (columns) is supported")
    f = np.asarray(f, float)
    shape = f.shape
    F = np.asfortranarray(f.reshape(shape[0], -1) if f.ndim > 1 else f[:, None])
    g = np.ascontiguousarray(np.asarray(g, float).ravel())
    h = np.zeros(F.shape, order="F")
    lib = _lib.load()
    check(lib.bfe_convolve(F.shape[0], F.shape[1], ptr(F, ctypes.c_double), g.size, ptr(g, ctypes.c_double),
                           ptr(h, ctypes.c_double)))
    return h.reshape(shape) if f.ndim > 1 else h[:, 0]


def _pair_lists(tx, rx, mon_nds_of_step, trans_nds, trans_wts):
    ptr_, slot, w = [0], [], []
    for a, b in zip(tx, rx):
        mon = np.asarray(mon_nds_of_step[a]).ravel()
        sel = np.nonzero(np.isin(mon, np.asarray(trans_nds[b]).ravel()))[0]
        wt = np.ones(sel.size) if trans_wts is None or trans_wts[b] is None else \
            np.asarray(trans_wts[b], float).ravel()
        if wt.size != sel.size:
            raise SolverError("receiver %d has %d weights for %d monitored nodes" % (b, wt.size, sel.size))
        slot.extend(sel.tolist())
        w.extend(wt.tolist())
        ptr_.append(len(slot))
    return (np.asarray(ptr_, np.int64), np.asarray(slot, np.int64), np.asarray(w, float))


def fn_parse_to_fmc_gb300(tx, rx, mon_nds_of_step, dsps_of_step, trans_nds, trans_wts, in_sig):
    """fn_parse_to_fmc (subdoms/fn_run_main_model.m:239-256) on the GPU
    (0-based tx, rx per pair). dsps_of_step is
    a list of per-step (q, n_t) displacement arrays, or one (q, n_t, R) array
    (e.g. Plan.run_batched's history); returns time_data (n_t, n_pairs)."""
    if isinstance(dsps_of_step, np.ndarray) and dsps_of_step.ndim == 3:
        hist = np.asfortranarray(dsps_of_step)
    else:
        q = max(np.asarray(d).shape[0] for d in dsps_of_step)
        n_t = np.asarray(dsps_of_step[0]).shape[1]
        hist = np.zeros((q, n_t, len(dsps_of_step)), order="F")
        for r, d in enumerate(dsps_of_step):
            hist[: np.asarray(d).shape[0], :, r] = d
    q, n_t, R = hist.shape
    p_, s_, w_ = _pair_lists(tx, rx, mon_nds_of_step, trans_nds, trans_wts)
    txa = np.ascontiguousarray(np.asarray(tx, np.int64))
    g = np.ascontiguousarray(np.asarray(in_sig, float).ravel()) if in_sig is not None else np.zeros(0)
    out = np.zeros((n_t, len(txa)), order="F")
    lib = _lib.load()
    check(lib.bfe_fmc_gather(q, n_t, R, ptr(hist, ctypes.c_double), len(txa), ptr(txa, ctypes.c_int64),
                             ptr(p_, ctypes.c_int64), ptr(s_, ctypes.c_int64), ptr(w_, ctypes.c_double),
                             g.size, ptr(g, ctypes.c_double) if g.size else None, ptr(out, ctypes.c_double)))
    return out


def fmc_from_device_history(d_hist, q, n_t, R, tx, rx_slots, rx_weights, in_sig, d_out, stream):
    """FMC time data from a device history (torch tensor laid out
    [R][n_t][q]) into d_out ([n_pairs][n_t]): rx_slots / rx_weights are one
    list per pair of history slots and weights."""
    p_ = np.zeros(len(tx) + 1, np.int64)
    p_[1:] = np.cumsum([len(x) for x in rx_slots])
    s_ = np.ascontiguousarray(np.concatenate([np.asarray(x, np.int64) for x in rx_slots]))
    w_ = np.ascontiguousarray(np.concatenate([np.asarray(x, float) for x in rx_weights]))
    txa = np.ascontiguousarray(np.asarray(tx, np.int64))
    g = np.ascontiguousarray(np.asarray(in_sig, float).ravel()) if in_sig is not None else np.zeros(0)
    lib = _lib.load()
    check(lib.bfe_fmc_gather_device(q, n_t, R, ctypes.c_void_p(d_hist.data_ptr()), len(txa),
                                    ptr(txa, ctypes.c_int64), ptr(p_, ctypes.c_int64), ptr(s_, ctypes.c_int64),
                                    ptr(w_, ctypes.c_double), g.size, ptr(g, ctypes.c_double) if g.size else None,
                                    ctypes.c_void_p(d_out.data_ptr()), ctypes.c_void_p(int(stream))))


def fn_convert_disps_to_forces_v2_gb300(K_sub, C_sub, M_sub, time_step, disp_inp, lyrs, in_or_out, solver_mode):
    """fn_convert_disps_to_forces_v2 (code/fn_convert_disps_to_forces_v2.m:1-31)
    on the GPU: returns (force_inp, force_set, force_in_set, force_out_set)
    like the reference."""
    if in_or_out not in ("in", "out"):
        raise SolverError("in_or_out must be 'in' or 'out'")
    modes = {VEL_CURRENT: _lib.BFE_MODE_VEL_CURRENT, VEL_LAST_HALF: _lib.BFE_MODE_VEL_LAST_HALF}
    if solver_mode not in modes:
        raise SolverError("unknown solver_mode %r" % (solver_mode,))
    lyrs = np.ascontiguousarray(np.asarray(lyrs).ravel().astype(np.int32))
    d = np.asfortranarray(np.asarray(disp_inp, float))
    n, n_t = d.shape
    Ks, k_ = _csr_view(K_sub, "K")
    Cs, c_ = _csr_view(C_sub, "C")
    Ms, m_ = _csr_view(M_sub, "M")
    force_in_set = lyrs == 2
    force_out_set = lyrs == 3
    force_set = force_in_set | force_out_set
    nf = int(force_set.sum())
    rows = np.zeros(max(n, 1), np.int64)
    out = np.zeros((nf, n_t), order="F")
    n_force = ctypes.c_int64()
    lib = _lib.load()
    check(lib.bfe_disps_to_forces(ctypes.byref(Ks), ctypes.byref(Cs), ctypes.byref(Ms), float(time_step), n_t,
                                  ptr(d, ctypes.c_double), ptr(lyrs, ctypes.c_int32), 0 if in_or_out == "in" else 1,
                                  modes[solver_mode], ctypes.byref(n_force), ptr(rows, ctypes.c_int64),
                                  ptr(out, ctypes.c_double) if nf else None))
    return out, force_set, force_in_set, force_out_set
