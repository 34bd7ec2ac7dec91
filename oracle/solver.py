"""Explicit time-marching restatements (FP64) - oracle only.

explicit_dynamic_solver_v6 follows code/internal/fn_explicit_dynamic_solver_v6.m
and explicit_dynamic_solver_v5 follows fn_explicit_dynamic_solver_v5.m. Index
arguments are 1-based like the reference's. The operators A, B, D of v6 are
applied as u = P^-1 (A' f + B' u_-1 + D' u_-2) with one sparse LU of
P = I + dt/2 M^-1 C, which is the same arithmetic as the reference's
precomputed P \\ (...) products (v6.m:136-138) up to FP64 rounding.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

VEL_LAST_HALF = "vel at last half time step"     # v6.m:131
VEL_CURRENT = "vel at curent time step"          # v6.m:135 (sic)
DISP_FIELD_TYPES = ("mean(u1)", "mean(u2)", "mean(u3)", "curl(u)", "div(u)", "raw(u)")  # v6.m:64-69


class SolverError(RuntimeError):
    pass


def _ti_start(forcing_indices, forcing_functions, disp_indices, disp_functions):
    """v6.m:163-169: first time index (1-based) with any non-zero input."""
    ti = np.inf
    if forcing_indices is not None and len(forcing_indices):
        nz = np.nonzero(np.abs(np.atleast_2d(forcing_functions)).sum(0))[0]
        if nz.size == 0:
            return None
        ti = min(nz.min() + 1, ti)
    if disp_indices is not None and len(disp_indices):
        nz = np.nonzero(np.abs(np.atleast_2d(disp_functions)).sum(0))[0]
        if nz.size == 0:
            return None
        ti = min(nz.min() + 1, ti)
    return None if np.isinf(ti) else int(ti)


def _forcing_column(F, ti, p):
    """f(forcing_indices) = forcing_functions(:, ti): one row broadcasts to
    every forced DOF, p rows assign row-wise (duplicate indices: last wins,
    like MATLAB indexed assignment); any other row count is an error."""
    col = F[:, ti - 1]
    if col.size == p:
        return col
    if col.size == 1:
        return col[0]
    raise SolverError("forcing_functions must have 1 or %d rows, got %d" % (p, col.size))


def lumped_mass(M):
    """sum(M).' (v6.m:122-123): column sums of M."""
    return np.asarray(M.sum(axis=0)).ravel()


def form_operators(K, C, M, dt, solver_mode):
    """Return (Pfactor, Aprime_diag, Bprime, Dprime) with
    u = P^-1 (A' f + B' u_-1 + D' u_-2) (v6.m:130-139)."""
    n = K.shape[0]
    m = lumped_mass(M)
    inv_m = 1.0 / m
    Minv = sp.diags(inv_m)
    I = sp.identity(n, format="csr")
    if solver_mode == VEL_LAST_HALF:
        return None, dt ** 2 * inv_m, (2 * I - dt * (Minv @ C) - dt ** 2 * (Minv @ K)).tocsr(), \
            (dt * (Minv @ C) - I).tocsr()
    if solver_mode == VEL_CURRENT:
        G = (dt / 2 * (Minv @ C)).tocsr()
        P = (I + G).tocsc()
        if G.nnz == 0 or (abs(G - sp.diags(G.diagonal())).sum() == 0):
            Pf = ("diag", P.diagonal())
        else:
            Pf = ("lu", spla.splu(P))
        return Pf, dt ** 2 * inv_m, (2 * I - dt ** 2 * (Minv @ K)).tocsr(), (-I + G).tocsr()
    # v6 leaves A, B, D undefined for any other string and fails at first use
    raise SolverError("unknown solver_mode %r (v6 accepts %r or %r)" % (solver_mode, VEL_LAST_HALF, VEL_CURRENT))


def _apply_pinv(Pf, r):
    if Pf is None:
        return r
    kind, obj = Pf
    if kind == "diag":
        return r / obj
    return obj.solve(r)


def explicit_dynamic_solver_v6(K, C, M, time, forcing_indices, forcing_functions,
                               disp_indices, disp_functions, history_indices,
                               field_output_every_n_frames, use_gpu_if_present=1,
                               field_output_type="KE", solver_mode=VEL_CURRENT,
                               solver_precision="double"):
    """fn_explicit_dynamic_solver_v6.m:1-221 (CPU path, FP64).

    Returns (history_output (q, n_t), field_output (n, n_frames) or None,
    force_output (None: v6's prescribed-displacement path is broken in the
    reference, v6.m:191 reads an undefined u_previous), field_output_time).
    """
    if K.shape[0] != K.shape[1]:
        raise SolverError("K must be square matrix")
    if C.shape[0] != C.shape[1]:
        raise SolverError("C must be square matrix")
    if M.shape[0] != M.shape[1]:
        raise SolverError("M must be square matrix")
    field_is_vel = field_output_type not in DISP_FIELD_TYPES
    time = np.asarray(time, float).ravel()
    nt = time.size
    ndf = K.shape[0]
    dt = time[1] - time[0]
    hist_idx = None if history_indices is None or len(history_indices) == 0 else \
        np.asarray(history_indices, np.int64).ravel() - 1
    hist = None if hist_idx is None else np.zeros((hist_idx.size, nt))
    if disp_indices is not None and len(disp_indices):
        raise SolverError("prescribed displacements: v6 reads undefined u_previous (v6.m:191)")
    if np.isinf(field_output_every_n_frames):
        fo_ti = np.zeros(0, np.int64)
        fld, fld_t = None, None
    else:
        fo_ti = np.arange(1, nt + 1, int(field_output_every_n_frames))
        fld = np.zeros((ndf, fo_ti.size))
        fld_t = np.zeros(fo_ti.size)
    Pf, Ad, Bp, Dp = form_operators(K, C, M, dt, solver_mode)
    u1 = np.zeros(ndf)
    u2 = np.zeros(ndf)
    f = np.zeros(ndf)
    frc_idx = None
    if forcing_indices is not None and len(forcing_indices):
        frc_idx = np.asarray(forcing_indices, np.int64).ravel() - 1
        F = np.atleast_2d(np.asarray(forcing_functions, float))
    ti0 = _ti_start(forcing_indices, forcing_functions, disp_indices, disp_functions)
    if ti0 is None:
        return hist, fld, None, fld_t
    frame_of = {int(t): k for k, t in enumerate(fo_ti)}
    for ti in range(ti0, nt + 1):
        if frc_idx is not None:
            f[frc_idx] = _forcing_column(F, ti, frc_idx.size)            # v6.m:182
        r = Ad * f + Bp @ u1 + Dp @ u2                                  # v6.m:185
        u = _apply_pinv(Pf, r)
        if hist is not None:
            hist[:, ti - 1] = u[hist_idx]                               # v6.m:196
        k = frame_of.get(ti)
        if k is not None:                                               # v6.m:200-208
            fld_t[k] = time[ti - 1]
            fld[:, k] = (u - u1) / dt if field_is_vel else u
        u2 = u1
        u1 = u
    return hist, fld, None, fld_t


def explicit_dynamic_solver_v5(K, C, M, time, forcing_indices, forcing_functions,
                               disp_indices, disp_functions, history_indices,
                               field_output_every_n_frames, use_gpu_if_present=1):
    """fn_explicit_dynamic_solver_v5.m:1-205 (CPU path, FP64).

    acceleration -> velocity -> displacement (v5.m:150-156); the history is u
    and the field output is always the velocity (v5.m:173-177).
    """
    time = np.asarray(time, float).ravel()
    nt = time.size
    ndf = K.shape[0]
    if C.shape != (ndf, ndf):
        raise SolverError("C must be square matrix, same size as K")
    if M.shape != (ndf, ndf):
        raise SolverError("M must be square matrix, same size as K")
    dt = time[1] - time[0]
    hist_idx = None if history_indices is None or len(history_indices) == 0 else \
        np.asarray(history_indices, np.int64).ravel() - 1
    hist = None if hist_idx is None else np.zeros((hist_idx.size, nt))
    disp_idx = None
    frc_out = None
    if disp_indices is not None and len(disp_indices):
        disp_idx = np.asarray(disp_indices, np.int64).ravel() - 1
        Dd = np.atleast_2d(np.asarray(disp_functions, float))
        frc_out = np.zeros((disp_idx.size, nt))
        tmp = np.hstack([np.zeros((Dd.shape[0], 2)), Dd])
        accn = (tmp[:, 2:] - 2 * tmp[:, 1:-1] + tmp[:, :-2]) / dt ** 2   # v5.m:73-76
        same_dof = (disp_idx[:, None] == disp_idx[None, :]).astype(float)
    if np.isinf(field_output_every_n_frames):
        fo_ti = np.zeros(0, np.int64)
        fld, fld_t = None, None
    else:
        fo_ti = np.arange(1, nt + 1, int(field_output_every_n_frames))
        fld = np.zeros((ndf, fo_ti.size))
        fld_t = np.zeros(fo_ti.size)
    m = lumped_mass(M)
    inv_m = 1.0 / m
    u_prev = np.zeros(ndf)
    ud_prev = np.zeros(ndf)
    f = np.zeros(ndf)
    frc_idx = None
    if forcing_indices is not None and len(forcing_indices):
        frc_idx = np.asarray(forcing_indices, np.int64).ravel() - 1
        F = np.atleast_2d(np.asarray(forcing_functions, float))
    ti0 = _ti_start(forcing_indices, forcing_functions, disp_indices, disp_functions)
    if ti0 is None:
        return hist, fld, frc_out, fld_t
    frame_of = {int(t): k for k, t in enumerate(fo_ti)}
    K = K.tocsr()
    C = C.tocsr()
    for ti in range(ti0, nt + 1):
        if frc_idx is not None and ti <= F.shape[1]:                     # v5.m:145-147
            f[frc_idx] = _forcing_column(F, ti, frc_idx.size)
        udd = inv_m * (f - K @ u_prev - C @ ud_prev)                     # v5.m:150
        ud = ud_prev + dt * udd                                          # v5.m:153
        u = u_prev + dt * ud                                             # v5.m:156
        if disp_idx is not None:                                         # v5.m:159-162
            u[disp_idx] = Dd[:, ti - 1]
            # diag_M(d, d) * accn: repeated DOFs in d make diag_M(d, d) a
            # block of equal masses, so each entry sums the accelerations of
            # every entry of the same DOF
            frc_out[:, ti - 1] = m[disp_idx] * (same_dof @ accn[:, ti - 1]) + K[disp_idx] @ u_prev
        if hist is not None:
            hist[:, ti - 1] = u[hist_idx]
        k = frame_of.get(ti)
        if k is not None:
            fld_t[k] = time[ti - 1]
            fld[:, k] = ud
        u_prev = u
        ud_prev = ud
    return hist, fld, frc_out, fld_t


def amplification_matrix_max_ev(M, C, K, dt, solver_mode=VEL_LAST_HALF):
    """tests/fn_amplification_matrix.m:1-41 - spectral radius of the
    two-step amplification matrix (dense eig, small models)."""
    n = K.shape[0]
    m = lumped_mass(M)
    Minv = np.diag(1.0 / m)
    Kd, Cd = K.toarray(), C.toarray()
    I = np.eye(n)
    if solver_mode == VEL_LAST_HALF:
        B1 = 2 * I - dt * Minv @ Cd - dt ** 2 * Minv @ Kd
        B2 = dt * Minv @ Cd - I
    else:
        B1 = 2 * I - dt ** 2 * Minv @ Kd
        B2 = -I + dt / 2 * Minv @ Cd
        B3 = I + dt / 2 * Minv @ Cd
        B1 = np.linalg.solve(B3, B1)
        B2 = np.linalg.solve(B3, B2)
    A = np.block([[B1, B2], [I, np.zeros((n, n))]])
    return np.abs(np.linalg.eigvals(A)).max()
