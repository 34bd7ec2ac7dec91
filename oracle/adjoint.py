"""FP64 discrete adjoint of the v6 time march - oracle only.

The reference has no adjoint; this restates the gradient of an A-scan misfit
for the v6 recurrence (code/internal/fn_explicit_dynamic_solver_v6.m:135-138,
'vel at curent time step'), written with the mass-weighted matrices

    R_t = A u_t - B u_{t-1} - E u_{t-2} - dt^2 f_t = 0,   t = t0 .. N-1
    A = M + dt/2 C,  B = 2 M - dt^2 K,  E = -M + dt/2 C

(u = P^-1 (A' f + B' u_{t-1} + D' u_{t-2}) multiplied through by M). With the
misfit J = 1/2 sum_t |S u_t - d_t|^2 the adjoint states satisfy

    A lam_t = B lam_{t+1} + E lam_{t+2} + S'(S u_t - d_t),  lam_N = lam_{N+1} = 0

(A, B, E are symmetric), and for per-element stiffness scales s_e
(K = sum_e s_e K_e) and densities rho_e (M = sum rho_e Mh_e, C = sum rho_e Ch_e)

    dJ/ds_e   = -dt^2 sum_t lam_t' K_e u_{t-1}
    dJ/drho_e = -sum_t lam_t' [Mh_e (u_t - 2 u_{t-1} + u_{t-2}) + dt/2 Ch_e (u_t - u_{t-2})]

(element-local contractions over the element's DOFs).
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from .solver import _ti_start


def element_data_cpe3(nds, els, el_abs, D, rho, gl, dof_to_use=(1, 2), damping_power_law=3,
                      max_damping=3.1415e7, max_stiffness_reduction=0.01):
    """Per-element unit-scale stiffness K_e (with the absorbing grading of
    fn_build_global_matrices_v5.m:116), lumped mass and damping per unit
    density (:115), and 0-based global DOF map, for CPE3 elements."""
    from .elements import el_CPE3
    K, _, M, ln, ld = el_CPE3(nds, els, D, rho, list(dof_to_use))
    a = np.asarray(el_abs, float)[:, None, None]
    K = K * np.exp(np.log(max_stiffness_reduction) * a ** (damping_power_law + 1))
    mh = np.einsum("eii->ei", M) / rho
    ch = mh * (np.asarray(el_abs, float)[:, None] ** damping_power_law * max_damping)
    dof = gl[els[:, ln - 1] - 1, ld - 1] - 1
    return K, mh, ch, dof


def _assemble(ke, mh, ch, dof, n, s, rho_e):
    e = np.repeat(np.arange(dof.shape[0]), dof.shape[1] ** 2)
    r = np.repeat(dof, dof.shape[1], axis=1).ravel()
    c = np.tile(dof, (1, dof.shape[1])).ravel()
    K = sp.csr_matrix(((ke * s[:, None, None]).transpose(0, 2, 1).ravel(), (r, c)), shape=(n, n))
    m = np.zeros(n)
    np.add.at(m, dof.ravel(), (mh * rho_e[:, None]).ravel())
    cc = np.zeros(n)
    np.add.at(cc, dof.ravel(), (ch * rho_e[:, None]).ravel())
    return K, m, cc


def forward(K, m, c, dt, n_t, frc_idx, F, ti0):
    """All states u_t (n, n_t) of one source, v6 'vel at curent time step'
    (code/internal/fn_explicit_dynamic_solver_v6.m:135-138, 185), written
    with the mass-weighted matrices of this module's header."""
    n = K.shape[0]
    A = m + dt / 2 * c
    E = -m + dt / 2 * c
    U = np.zeros((n, n_t))
    f = np.zeros(n)
    u1 = np.zeros(n)
    u2 = np.zeros(n)
    for t in range(ti0, n_t):
        f[frc_idx] = F[:, t] if F.shape[0] == len(frc_idx) else F[0, t]
        u = (dt ** 2 * f + 2 * m * u1 - dt ** 2 * (K @ u1) + E * u2) / A
        U[:, t] = u
        u2, u1 = u1, u
    return U


def misfit_and_gradient(ke, mh, ch, dof, n, dt, n_t, srcs, F, hist_idx, observed,
                        s=None, rho_e=None):
    """J and (dJ/ds, dJ/drho) summed over sources (0-based indices).

    srcs: list of R forced-DOF arrays; F: (rows, n_t) shared signal;
    observed: (q, n_t, R)."""
    n_el = dof.shape[0]
    s = np.ones(n_el) if s is None else s
    rho_e = np.ones(n_el) if rho_e is None else rho_e
    K, m, c = _assemble(ke, mh, ch, dof, n, s, rho_e)
    A = m + dt / 2 * c
    E = -m + dt / 2 * c
    J = 0.0
    gs = np.zeros(n_el)
    gr = np.zeros(n_el)
    F = np.atleast_2d(F)
    ti0 = _ti_start([0], F, [], [])
    if ti0 is None:
        return 0.0, gs, gr
    ti0 -= 1
    for r, fi in enumerate(srcs):
        U = forward(K, m, c, dt, n_t, np.asarray(fi), F, ti0)
        res = U[hist_idx] - observed[:, :, r]
        res[:, :ti0] = 0.0
        J += 0.5 * (res ** 2).sum()
        l1 = np.zeros(n)          # lam_{t+1}
        l2 = np.zeros(n)          # lam_{t+2}
        for t in range(n_t - 1, ti0 - 1, -1):
            g = np.zeros(n)
            np.add.at(g, hist_idx, res[:, t])
            lam = (2 * m * l1 - dt ** 2 * (K @ l1) + E * l2 + g) / A
            um = U[:, t - 1] if t - 1 >= ti0 else np.zeros(n)
            umm = U[:, t - 2] if t - 2 >= ti0 else np.zeros(n)
            ut = U[:, t]
            le = lam[dof]
            gs += -dt ** 2 * np.einsum("ei,eij,ej->e", le, ke, um[dof])
            gr += -np.einsum("ei,ei->e", le, mh * (ut - 2 * um + umm)[dof] + dt / 2 * ch * (ut - umm)[dof])
            l2, l1 = l1, lam
    return J, gs, gr


def misfit(ke, mh, ch, dof, n, dt, n_t, srcs, F, hist_idx, observed, s=None, rho_e=None):
    """J only (for finite differences)."""
    n_el = dof.shape[0]
    s = np.ones(n_el) if s is None else s
    rho_e = np.ones(n_el) if rho_e is None else rho_e
    K, m, c = _assemble(ke, mh, ch, dof, n, s, rho_e)
    F = np.atleast_2d(F)
    ti0 = _ti_start([0], F, [], []) - 1
    J = 0.0
    for r, fi in enumerate(srcs):
        U = forward(K, m, c, dt, n_t, np.asarray(fi), F, ti0)
        res = U[hist_idx] - observed[:, :, r]
        res[:, :ti0] = 0.0
        J += 0.5 * (res ** 2).sum()
    return J
