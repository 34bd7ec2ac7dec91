"""fn_BristolFE_v2 and fn_get_field_output restatements (FP64) - oracle only."""
import numpy as np

from .assembly import build_global_matrices_v5, set_default_fields
from .solver import (VEL_CURRENT, explicit_dynamic_solver_v5,
                     explicit_dynamic_solver_v6)

DEFAULT_CORE_OPTIONS = dict(                    # fn_BristolFE_v2.m:22-30
    use_gpu_if_available=1,
    global_matrix_builder_version="v5",
    dynamic_solver_version="v6",
    solver_mode=VEL_CURRENT,
    field_output_type="KE",
)
DEFAULT_ENTRY_OPTIONS = dict(                   # fn_FE_entry_point.m:23-35
    solver="BristolFE",
    damping_power_law=3,
    max_damping=3.1415e7,
    max_stiffness_reduction=0.01,
    solver_precision="double",
    field_output_every_n_frames=np.inf,
    dof_to_use=[],
)


def nds_and_dfs_to_gi(nds, dfs, gl_lookup):
    """fn_BristolFE_v2.m:159-168 - (node, dof) pairs (1-based) to 1-based
    global indices; pairs that map to 0 are dropped, ``valid`` marks kept ones."""
    nds = np.asarray(nds, np.int64).ravel()
    dfs = np.asarray(dfs, np.int64).ravel()
    gi = gl_lookup[nds - 1, dfs - 1]      # IndexError like MATLAB's out-of-range
    valid = gi > 0
    return gi[valid], nds[valid], dfs[valid], valid


def _mask_rows(a, mask):
    """a(mask, :) with MATLAB's logical indexing: a mask shorter than the
    rows selects among the first rows (fn_BristolFE_v2.m:82-84 applies a
    step's validity mask to forces that steps{1}.load.wts may have given
    more rows); a true beyond the last row is an index error."""
    idx = np.nonzero(np.asarray(mask, bool).ravel())[0]
    if idx.size and idx.max() >= a.shape[0]:
        raise IndexError("logical index exceeds the %d rows" % a.shape[0])
    return a[idx]


def _grow_rows(valid, values, nt):
    """res.dsps(valid, :) = values on an unset field (fn_BristolFE_v2.m:127):
    MATLAB sizes the new array to the last true index of the mask."""
    rows = int(np.nonzero(valid)[0].max()) + 1 if valid.any() else 0
    out = np.zeros((rows, nt))
    out[valid[:rows]] = values
    return out


def BristolFE_v2(mod, matls, steps, fe_options=None):
    """fn_BristolFE_v2.m:1-157. Returns (res, mats)."""
    opt = set_default_fields(fe_options, DEFAULT_CORE_OPTIONS)
    opt = set_default_fields(opt, DEFAULT_ENTRY_OPTIONS)
    mod = dict(mod)
    if "el_typ_i" not in mod:
        mod["el_typ_i"] = [matls[m - 1]["el_typ"] for m in mod["el_mat_i"]]
    if "el_abs_i" not in mod:
        mod["el_abs_i"] = np.zeros(len(mod["el_mat_i"]))
    K, C, M, gl = build_global_matrices_v5(mod["nds"], mod["els"], mod["el_mat_i"],
                                           mod["el_abs_i"], mod["el_typ_i"], matls, opt)
    mats = dict(K=K, C=C, M=M, gl_lookup=gl)
    if not isinstance(steps, (list, tuple)):
        steps = [steps]
    res = []
    for s, st in enumerate(steps):
        r = {}
        load = st["load"]
        if "time" not in load:
            res.append(r)
            continue
        t = np.asarray(load["time"], float).ravel()
        nt = t.size
        if "frcs" in load:
            frc_gi, _, _, valid_f = nds_and_dfs_to_gi(load["frc_nds"], load["frc_dfs"], gl)
            frcs = np.atleast_2d(np.asarray(load["frcs"], float))
            if "wts" in steps[0]["load"]:              # steps{1} used for all (:79)
                frcs = np.asarray(steps[0]["load"]["wts"], float).reshape(-1, 1) @ frcs
            if frcs.shape[0] > 1:
                frcs = _mask_rows(frcs, valid_f)
        else:
            frc_gi, frcs = np.zeros(0, np.int64), None
        dsp_gi, dsps = np.zeros(0, np.int64), None
        if "dsps" in load:
            dsp_gi, _, _, r["valid_appl_dsps"] = nds_and_dfs_to_gi(load["dsp_nds"], load["dsp_dfs"], gl)
            dsps = np.atleast_2d(np.asarray(load["dsps"], float))
            if "wts" in steps[0]["load"]:
                dsps = np.asarray(steps[0]["load"]["wts"], float).reshape(-1, 1) @ dsps
            if dsps.shape[0] > 1:
                dsps = _mask_rows(dsps, r["valid_appl_dsps"])
        mon = st.get("mon", {})
        if "nds" in mon:
            hist_gi, _, _, r["valid_mon_dsps"] = nds_and_dfs_to_gi(mon["nds"], mon["dfs"], gl)
        else:
            hist_gi = np.zeros(0, np.int64)
        if opt["dynamic_solver_version"] == "v5":
            h, fld, mf, r["fld_time"] = explicit_dynamic_solver_v5(
                K, C, M, t, frc_gi, frcs, dsp_gi, dsps, hist_gi,
                opt["field_output_every_n_frames"], opt["use_gpu_if_available"])
        else:
            h, fld, mf, r["fld_time"] = explicit_dynamic_solver_v6(
                K, C, M, t, frc_gi, frcs, dsp_gi, dsps, hist_gi,
                opt["field_output_every_n_frames"], opt["use_gpu_if_available"],
                opt["field_output_type"], opt["solver_mode"], opt["solver_precision"])
        if "nds" in mon:
            r["dsps"] = _grow_rows(r["valid_mon_dsps"], h if h is not None else np.zeros((0, nt)), nt)
            r["dsp_gi"] = hist_gi
        else:
            r["dsps"], r["dsp_gi"] = None, None
        if "dsps" in load:
            r["frcs"] = _grow_rows(r["valid_appl_dsps"], mf, nt)
            r["frc_gi"] = frc_gi
        else:
            r["frcs"], r["frc_gi"] = None, None
        r["fld"] = get_field_output(fld, mod, mats, opt["field_output_type"]) if fld is not None else None
        r["raw_fld"] = fld
        res.append(r)
    return res, mats


def _global_to_nodal(gv, gl_lookup):
    """fn_get_field_output.m:109-118 -> (n_nodes, n_frames, n_dof_cols)."""
    nv = np.zeros((gl_lookup.shape[0], gv.shape[1], gl_lookup.shape[1]))
    for i in range(gl_lookup.shape[1]):
        j = gl_lookup[:, i]
        valid = j > 0
        jj = np.where(valid, j, 1) - 1
        nv[:, :, i] = gv[jj, :] * valid[:, None]
    return nv


def _average_over_nodes(nv, els):
    """fn_get_field_output.m:121-135."""
    els = np.asarray(els)
    sz = nv.shape
    nv = nv.reshape(sz[0], -1)
    ev = np.zeros((els.shape[0], nv.shape[1]))
    n = np.zeros((els.shape[0], 1))
    for i in range(els.shape[1]):
        j = els[:, i]
        valid = j > 0
        jj = np.where(valid, j, 1) - 1
        ev += nv[jj, :] * valid[:, None]
        n += valid[:, None]
    ev = ev / n
    return ev.reshape((els.shape[0],) + sz[1:])


def element_centres(nds, els):
    """code/fn_calc_element_centres.m:1-18: mean of each element's nodes."""
    els = np.asarray(els)
    c = np.zeros((els.shape[0], nds.shape[1]))
    n = np.zeros((els.shape[0], 1))
    for i in range(els.shape[1]):
        v = els[:, i] > 0
        j = np.where(v, els[:, i], 1) - 1
        n += v[:, None]
        c += nds[j, :] * v[:, None]
    return c / n


def _unit_vecs_div(mod):
    """fn_get_field_output.m:84-98: unit vectors from each element's centre to
    its nodes; all zero for elements with an unused node column."""
    nds, els = mod["nds"], np.asarray(mod["els"])
    uv = np.zeros(els.shape + (nds.shape[1],))
    valid = np.ones(els.shape[0], bool)
    for i in range(els.shape[1]):
        valid &= els[:, i] > 0
        j = np.where(els[:, i] > 0, els[:, i], 1) - 1
        uv[:, i, :] = nds[j, :]
    uv = uv - element_centres(nds, els)[:, None, :]
    uv = uv / np.sqrt((uv ** 2).sum(axis=2, keepdims=True))
    uv[~valid] = 0.0
    return uv


def _unit_vecs_curl(mod):
    """fn_get_field_output.m:100-104: div vectors rotated by 90 degrees."""
    uv = _unit_vecs_div(mod)
    return np.stack([uv[:, :, 1], -uv[:, :, 0]], axis=2)


def get_field_output(f_out, mod, mats, field_output_type="sqrt(KE)"):
    """fn_get_field_output.m:1-80 ('sqrt(KE)' default, mean(ui)/mean(vi),
    div/curl, raw)."""
    t = field_output_type
    if t in ("mean(u1)", "mean(u2)", "mean(u3)", "mean(v1)", "mean(v2)", "mean(v3)"):
        nv = _global_to_nodal(f_out, mats["gl_lookup"])
        k = int(t[6])
        return _average_over_nodes(nv[:, :, k - 1], mod["els"])
    if t in ("raw(u)", "raw(v)"):
        return t
    if t in ("curl(u)", "div(u)", "curl(v)", "div(v)"):
        nv = _global_to_nodal(f_out, mats["gl_lookup"])                 # :34
        if t.startswith("div"):
            uv = _unit_vecs_div(mod)                                    # :49-50
        else:
            if mod["nds"].shape[1] > 2:                                 # :52-54
                raise ValueError("Cannot output curl for 3D models")
            uv = _unit_vecs_curl(mod)
        els = np.asarray(mod["els"])
        v = np.zeros((els.shape[0], f_out.shape[1]))                    # :58-63
        d = uv.shape[2]
        for i in range(els.shape[1]):
            j = np.where(els[:, i] > 0, els[:, i], 1) - 1
            v = v + (nv[j, :, :d] * uv[:, i, None, :]).sum(axis=2)
        return v
    dM = mats["M"].diagonal()
    KE_g = np.abs(f_out ** 2 * dM[:, None]) / 2                       # :64-67
    KE_n = _global_to_nodal(KE_g, mats["gl_lookup"]).sum(axis=2)        # :70-71
    return np.sqrt(_average_over_nodes(KE_n, mod["els"]))              # :74
