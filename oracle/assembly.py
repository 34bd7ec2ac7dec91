"""Global assembly restatement (fn_build_global_matrices_v5) - oracle only."""
import numpy as np
import scipy.sparse as sp

from .elements import ELEMENTS

DEFAULT_BUILD_OPTIONS = dict(         # fn_build_global_matrices_v5.m:26-33
    dof_to_use=[],
    damping_power_law=3,
    max_damping=3.1415e7,
    max_stiffness_reduction=0.01,
    interface_damping_factor=0,
)


def set_default_fields(opts, defaults):
    """fn_set_default_fields.m:18-26 - add missing keys only."""
    out = dict(opts or {})
    for k, v in defaults.items():
        if k not in out:
            out[k] = v
    return out


def find_dof_in_use_and_max_dof_per_el(unique_typs, dof_to_use):
    """fn_find_dof_in_use_and_max_dof_per_el.m:1-21."""
    dof_in_use = []
    max_dof_per_el = 0
    for t in unique_typs:
        _, _, _, _, loc_df = ELEMENTS[t](None, None, None, None, dof_to_use)
        dof_in_use.extend(loc_df.tolist())
        max_dof_per_el = max(max_dof_per_el, len(loc_df))
    return np.unique(np.array(dof_in_use, dtype=np.int64)), max_dof_per_el


def _material(matls, m):
    """D and rho of material m (1-based; 0 = none) (v5.m:85-102)."""
    if m > 0:
        mt = matls[m - 1]
        D = np.asarray(mt["D"], float)
        rho = mt["density"] if "density" in mt else mt["rho"]
    else:
        D = np.zeros(()) ; rho = 0.0
    if D.ndim == 2 and D.shape == (3, 3):      # legacy 3x3 plane matrix (v5.m:99-102)
        D6 = np.zeros((6, 6))
        idx = [0, 1, 5]
        D6[np.ix_(idx, idx)] = D
        D = D6
    return D, rho


def build_global_matrices_v5(nds, els, el_mat_i, el_abs_i, el_typ_i, matls, fe_options=None):
    """fn_build_global_matrices_v5.m:1-167.

    Returns (K, C, M, gl_lookup) with K, C, M as scipy CSR matrices over the
    reduced global DOFs and gl_lookup an (n_nodes, n_dof_cols) int array of
    1-based global indices (0 = unused), exactly as the reference numbers
    them: node-major, DOF-minor over max_df, compacted (v5.m:127-128,150-159).
    """
    opt = set_default_fields(fe_options, DEFAULT_BUILD_OPTIONS)
    els = np.asarray(els, dtype=np.int64)
    el_mat_i = np.asarray(el_mat_i, dtype=np.int64).ravel()
    el_abs_i = np.asarray(el_abs_i, float).ravel()
    typ = np.array(list(el_typ_i), dtype=object)
    if el_mat_i.size != els.shape[0]:
        raise ValueError("Length of element materials vector must equal number of elements")
    unique_typs = sorted(set(typ.tolist()))                       # v5.m:51
    unique_df, max_el_df = find_dof_in_use_and_max_dof_per_el(unique_typs, opt["dof_to_use"])
    max_df = int(unique_df.max())                                 # v5.m:54
    no_nds = nds.shape[0]
    total_dof = no_nds * max_df
    gi_all, gj_all, kv, mv, cv = [], [], [], [], []
    p = opt["damping_power_law"]
    for t in unique_typs:                                          # v5.m:70
        el_i = typ == t
        for m in np.unique(el_mat_i[el_i]):                        # v5.m:75-78
            el_i2 = (el_mat_i == m) & el_i
            if not el_i2.any():
                continue
            D, rho = _material(matls, int(m))
            eK, eC, eM, loc_nd, loc_df = ELEMENTS[t](nds, els[el_i2], D, rho, opt["dof_to_use"])
            a = el_abs_i[el_i2][:, None, None]
            eC = eC + eM * a ** p * opt["max_damping"]             # v5.m:115
            eK = eK * np.exp(np.log(opt["max_stiffness_reduction"]) * a ** (p + 1))  # v5.m:116
            # K(gi(c), gi(r)) += el_K(r, c)  (v5.m:119-139 with meshgrid order)
            ge = (els[el_i2][:, loc_nd - 1] - 1) * max_df + loc_df - 1       # (n, ndf) 0-based
            ndf = len(loc_df)
            gi = np.broadcast_to(ge[:, None, :], (ge.shape[0], ndf, ndf))  # column dof c
            gj = np.broadcast_to(ge[:, :, None], (ge.shape[0], ndf, ndf))  # row dof r
            gi_all.append(gi.ravel()); gj_all.append(gj.ravel())
            kv.append(eK.ravel()); mv.append(eM.ravel()); cv.append(eC.ravel())
    gi = np.concatenate(gi_all); gj = np.concatenate(gj_all)
    shape = (total_dof, total_dof)
    K = sp.coo_matrix((np.concatenate(kv), (gi, gj)), shape=shape).tocsr()
    M = sp.coo_matrix((np.concatenate(mv), (gi, gj)), shape=shape).tocsr()
    C = sp.coo_matrix((np.concatenate(cv), (gi, gj)), shape=shape).tocsr()
    for X in (K, M, C):
        X.sum_duplicates()
        X.eliminate_zeros()               # MATLAB sparse keeps nonzeros only
    gl_nds = np.repeat(np.arange(1, no_nds + 1), max_df)          # v5.m:150-153
    gl_dofs = np.tile(np.arange(1, max_df + 1), no_nds)
    gl_nds, gl_dofs, K, M, C = reduce_global_matrices(gl_nds, gl_dofs, K, M, C)
    gl_lookup = create_fast_lookup(gl_nds, gl_dofs, no_nds, 0)
    if opt["interface_damping_factor"]:
        C = add_interface_damping(els, typ, K, C, M, gl_lookup, opt["interface_damping_factor"])
    return K, C, M, gl_lookup


def reduce_global_matrices(gl_nds, gl_dofs, *mats):
    """fn_reduce_global_matrices.m:1-22 - drop DOFs whose columns are all zero
    in every matrix."""
    valid = None
    for X in mats:
        v = np.asarray(abs(X).sum(axis=0)).ravel() > 0
        valid = v if valid is None else (valid | v)
    keep = np.nonzero(valid)[0]
    out = [X[keep][:, keep].tocsr() for X in mats]
    return (gl_nds[keep], gl_dofs[keep], *out)


def create_fast_lookup(gl_nds, gl_dofs, max_nds, max_dofs):
    """fn_create_fast_lookup.m:1-8 (1-based indices, 0 = absent)."""
    nr = max(int(gl_nds.max()) if gl_nds.size else 0, max_nds)
    nc = max(int(gl_dofs.max()) if gl_dofs.size else 0, max_dofs)
    lk = np.zeros((nr, nc), dtype=np.int64)
    lk[gl_nds - 1, gl_dofs - 1] = np.arange(1, gl_nds.size + 1)
    return lk


def add_interface_damping(els, el_typ_i, K, C, M, gl_lookup, factor=1):
    """fn_add_interface_damping.m:30-52: C(gi,gi) += M(gi,gi) * level on all
    DOFs of interface nodes, level = min(sqrt(diag K / diag M)) / pi^2 * factor."""
    dK = K.diagonal()
    dM = M.diagonal()
    with np.errstate(divide="ignore", invalid="ignore"):
        level = np.nanmin(np.sqrt(dK / dM)) / np.pi ** 2 * factor
    typ = np.array(list(el_typ_i), dtype=object)
    nd = np.asarray(els)[typ == "ASI2D2"]
    nd = nd[nd > 0]
    if nd.size == 0:
        return C
    gi = gl_lookup[nd - 1, :].ravel()
    gi = np.unique(gi[gi > 0]) - 1
    add = np.zeros(C.shape[0])
    add[gi] = dM[gi] * level
    return (C + sp.diags(add)).tocsr()
