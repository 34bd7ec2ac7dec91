"""FP64 CPU time march of the v6 path in C (oracle/c/cpu_march.c) - oracle only.

Operators are formed in FP64 exactly as fn_explicit_dynamic_solver_v6.m:122-139
(the exact P^-1 on the fluid-solid interface block comes from a dense inverse
of that block, which is what the reference's P \\ (...) computes), then the C
loop marches them on all host threads.
"""
import ctypes
import time as _time

import numpy as np
import scipy.sparse as sp

from . import cbuild
from .solver import VEL_CURRENT, VEL_LAST_HALF, lumped_mass

_lib = None


def _load():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(cbuild.build())
        _lib.cpu_threads.restype = ctypes.c_int
    return _lib


def threads():
    """OpenMP threads the C port uses (all host threads)."""
    return _load().cpu_threads()


class CpuOperator:
    """v6 operators (FP64) prepared for the C loop."""

    def __init__(self, K, C, M, dt, solver_mode=VEL_CURRENT):
        n = K.shape[0]
        m = lumped_mass(M)
        inv_m = 1.0 / m
        Minv = sp.diags(inv_m)
        I = sp.identity(n, format="csr")
        Cd = C.diagonal()
        Coff = (C - sp.diags(Cd)).tocsr()
        Coff.eliminate_zeros()
        self.acoef = dt ** 2 * inv_m
        if solver_mode == VEL_LAST_HALF:
            B = (2 * I - dt * (Minv @ C) - dt ** 2 * (Minv @ K)).tocsr()
            D = (dt * (Minv @ C) - I).tocsr()
            pinv = np.ones(n)
            irows = np.zeros(0, np.int64)
            Pi = sp.csr_matrix((0, n))
        elif solver_mode == VEL_CURRENT:
            B = (2 * I - dt ** 2 * (Minv @ K)).tocsr()
            D = (-I + dt / 2 * (Minv @ C)).tocsr()
            P = (I + dt / 2 * (Minv @ C)).tocsr()
            pinv = 1.0 / P.diagonal()
            irows = np.unique(np.concatenate(Coff.nonzero())).astype(np.int64)
            if irows.size:
                Pii = P[irows][:, irows].toarray()
                Zi = np.linalg.inv(Pii)
                Zi[np.abs(Zi) < 1e-300] = 0.0
                Pi = sp.csr_matrix((irows.size, n))
                Pi = sp.csr_matrix((Zi[np.nonzero(Zi)], (np.nonzero(Zi)[0], irows[np.nonzero(Zi)[1]])),
                                   shape=(irows.size, n))
            else:
                Pi = sp.csr_matrix((0, n))
        else:
            raise ValueError(solver_mode)
        self.n = n
        self.B = B
        diag_only = abs(D - sp.diags(D.diagonal())).sum() == 0
        self.D = None if diag_only else D
        self.dvec = D.diagonal()
        if diag_only:
            # fold diagonal D into B's loop as a separate vector via D CSR of the diagonal
            self.D = sp.diags(self.dvec).tocsr()
        self.pinv = pinv
        self.irows = irows
        self.Pi = Pi.tocsr()

    def march(self, time, frc_idx0, F, hist_idx0, every_n=0, field_is_vel=True, frames=False):
        """FP64 march of one source (0-based indices). F: (rows, n_t), rows 1 or p.

        Returns the q x n_t history; with frames=True returns (hist, fld,
        fld_time), fld n x n_frames holding a frame every every_n samples
        from the first (fn_explicit_dynamic_solver_v6.m:200-208)."""
        lib = _load()
        nt = len(time)
        F = np.atleast_2d(np.asarray(F, float))
        frc_idx0 = np.asarray(frc_idx0, np.int64)
        # last-wins dedupe of duplicate forced DOFs
        last = {}
        for e, d in enumerate(frc_idx0):
            last[int(d)] = e
        rows = np.array(sorted(last), np.int64)
        sigk = np.array([0 if F.shape[0] == 1 else last[d] for d in rows], np.int64)
        nz = np.nonzero(np.abs(F).sum(0))[0]
        ti0 = int(nz.min()) if (rows.size and nz.size) else nt
        sig = np.ascontiguousarray(F.T)
        hist_idx0 = np.asarray(hist_idx0, np.int64)
        q = hist_idx0.size
        hist = np.zeros((q, nt), order="F")
        every = int(every_n) if (frames and every_n and every_n > 0) else 0
        nf = (nt + every - 1) // every if every else 0
        fld = np.zeros((self.n, nf), order="F")
        fld_t = np.zeros(nf)
        tm = np.ascontiguousarray(np.asarray(time, float))
        dt = float(tm[1] - tm[0]) if nt > 1 else 1.0

        def P(a, t):
            return a.ctypes.data_as(ctypes.POINTER(t))
        B, D, Pi = self.B, self.D, self.Pi
        arrs = [B.indptr.astype(np.int64), B.indices.astype(np.int64), B.data.astype(np.float64),
                D.indptr.astype(np.int64), D.indices.astype(np.int64), D.data.astype(np.float64),
                Pi.indptr.astype(np.int64), Pi.indices.astype(np.int64), Pi.data.astype(np.float64)]
        c64, cd = ctypes.c_int64, ctypes.c_double
        st = lib.cpu_march(
            c64(self.n), P(arrs[0], c64), P(arrs[1], c64), P(arrs[2], cd),
            P(arrs[3], c64), P(arrs[4], c64), P(arrs[5], cd),
            P(self.acoef, cd), P(self.pinv, cd),
            c64(self.irows.size), P(self.irows, c64), P(arrs[6], c64), P(arrs[7], c64), P(arrs[8], cd),
            c64(nt), c64(ti0), c64(rows.size), P(rows, c64), P(sigk, c64), c64(sig.shape[1]),
            P(sig, cd), c64(q), P(hist_idx0, c64), P(hist, cd),
            c64(every), ctypes.c_int32(1 if field_is_vel else 0), cd(dt), P(tm, cd),
            P(fld, cd) if every else None, P(fld_t, cd) if every else None)
        if st != 0:
            raise RuntimeError("cpu_march failed")
        return (hist, fld, fld_t) if frames else hist


def time_march(op, time, frc_idx0, F, hist_idx0, min_seconds=0.0):
    """Run the march and return (hist, seconds)."""
    t0 = _time.perf_counter()
    h = op.march(time, frc_idx0, F, hist_idx0)
    return h, _time.perf_counter() - t0
