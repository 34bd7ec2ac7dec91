"""Sub-domain and FMC post-processing restatements (FP64) - oracle only.

Test infrastructure: the product's GPU versions are checked against these.
"""
import numpy as np
import scipy.sparse as sp

from .solver import VEL_CURRENT, VEL_LAST_HALF


def convert_disps_to_forces_v2(K_sub, C_sub, M_sub, time_step, disp_inp, lyrs, in_or_out, solver_mode):
    """code/fn_convert_disps_to_forces_v2.m:1-31: forces on layers 2 and 3 of
    a sub-domain that reproduce the given displacements; layers 3, 4 ('in')
    or 1, 2 ('out') are frozen. Returns (force_inp, force_set, force_in_set,
    force_out_set)."""
    lyrs = np.asarray(lyrs).ravel()
    force_in_set = lyrs == 2
    force_out_set = lyrs == 3
    force_set = force_in_set | force_out_set
    if in_or_out == "in":
        freeze = (lyrs == 3) | (lyrs == 4)
    elif in_or_out == "out":
        freeze = (lyrs == 1) | (lyrs == 2)
    else:
        raise ValueError("in_or_out must be 'in' or 'out'")          # switch falls through: freeze_set undefined
    d = np.array(disp_inp, float)
    d[freeze, :] = 0.0                                                  # :11
    m = np.asarray(M_sub.sum(axis=0)).ravel()                           # :12 spdiags(sum(M_sub).')
    tmp = np.hstack([np.zeros((d.shape[0], 2)), d])                     # :14
    accn = (tmp[:, 2:] - 2 * tmp[:, 1:-1] + tmp[:, :-2]) / time_step ** 2
    if solver_mode == VEL_LAST_HALF:
        vel = (tmp[:, 1:-1] - tmp[:, :-2]) / time_step                  # :18
    elif solver_mode == VEL_CURRENT:
        vel = (tmp[:, 2:] - tmp[:, :-2]) / (2 * time_step)              # :20
    else:
        raise ValueError("unknown solver_mode")
    disp = np.hstack([np.zeros((d.shape[0], 1)), d[:, :-1]])           # :22
    fs = np.nonzero(force_set)[0]
    force = m[fs, None] * accn[fs] + sp.csr_matrix(C_sub)[fs] @ vel + sp.csr_matrix(K_sub)[fs] @ disp
    return force, force_set, force_in_set, force_out_set


def convolve(f, g, dim=0):
    """code/internal/fn_convolve.m:22-33: FFT convolution with 2 * size(f, dim)
    points, truncated to the size of f (the linear convolution's first
    samples)."""
    f = np.asarray(f, float)
    g = np.asarray(g, float)
    n = 2 * f.shape[dim]
    F = np.fft.fft(f, n, axis=dim)
    G = np.fft.fft(g, n, axis=dim)
    if G.ndim < F.ndim:
        G = G.reshape(G.shape + (1,) * (F.ndim - G.ndim)) if dim == 0 else G
    h = np.fft.ifft(F * G, n, axis=dim).real
    return h[tuple(slice(0, s) for s in f.shape)]


def parse_to_fmc(tx, rx, mon_nds_of_step, dsps_of_step, trans_nds, trans_wts, in_sig):
    """subdoms/fn_run_main_model.m:239-256 (fn_parse_to_fmc): for each pair k
    the rows of step tx[k]'s monitored displacements whose node belongs to
    receiver rx[k], summed (or weighted by the receiver's wt), convolved with
    the input signal. tx, rx are 0-based; returns time_data (n_t, n_pairs)."""
    n_t = dsps_of_step[tx[0]].shape[1]
    out = np.zeros((n_t, len(tx)))
    for k, (a, b) in enumerate(zip(tx, rx)):
        sel = np.isin(np.asarray(mon_nds_of_step[a]).ravel(), np.asarray(trans_nds[b]).ravel())
        tmp = dsps_of_step[a][sel, :]
        w = trans_wts[b] if trans_wts is not None else None
        tmp = (np.asarray(w, float).ravel() @ tmp) if w is not None else tmp.sum(axis=0)
        out[:, k] = tmp
        if in_sig is not None and np.size(in_sig):
            out[:, k] = convolve(out[:, k], np.asarray(in_sig, float).ravel())
    return out
