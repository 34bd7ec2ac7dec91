"""The reference's entry function on the GPU path: the mirror of
fn_BristolFE_v2(mod, matls, steps, fe_options) (code/fn_BristolFE_v2.m:1-157).

Assembly runs on the host (``model.assemble``, the v5 builder with the
reference's DOF numbering); every load step marches on the GPU through one
plan that stays resident for all steps (the reference rebuilds its operators
for every step, fn_explicit_dynamic_solver_v6.m:122-159). Field frames are
reduced to element values on the device while the march runs. Steps that
share their time axis and monitors and need neither frames nor prescribed
displacements are marched together as one multi-right-hand-side run
(``batch_steps``, on by default); their results are identical to separate
runs up to rounding.
"""
import numpy as np
import scipy.sparse as sp

from . import model
from .field import FieldOutput, field_type_code
from .solver import V5, VEL_CURRENT, VEL_LAST_HALF, Plan, SolverError

DEFAULT_OPTIONS = dict(                      # fn_BristolFE_v2.m:22-30
    use_gpu_if_available=1,
    global_matrix_builder_version="v5",
    dynamic_solver_version="v6",
    solver_mode=VEL_CURRENT,
    field_output_type="KE",
)
DEFAULT_RUN_OPTIONS = dict(                  # fn_FE_entry_point.m:23-35, fn_build_global_matrices_v5.m:26-33
    damping_power_law=3,
    max_damping=3.1415e7,
    max_stiffness_reduction=0.01,
    interface_damping_factor=0,
    solver_precision="double",
    field_output_every_n_frames=np.inf,
    dof_to_use=[],
    batch_steps=True,
    assemble_on_gpu=True,
)


def _set_default_fields(opts, defaults):
    """fn_set_default_fields: add missing keys only."""
    out = dict(opts or {})
    for k, v in defaults.items():
        out.setdefault(k, v)
    return out


def nds_and_dfs_to_gi(nds, dfs, gl_lookup):
    """fn_BristolFE_v2.m:159-168: (node, dof) pairs (1-based) to 1-based
    global indices; pairs without a DOF are dropped and ``valid`` marks the
    kept ones."""
    nds = np.asarray(nds, np.int64).ravel()
    dfs = np.asarray(dfs, np.int64).ravel()
    gi = gl_lookup[nds - 1, dfs - 1]
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
    the array grows to the last valid row."""
    rows = int(np.nonzero(valid)[0].max()) + 1 if valid.any() else 0
    out = np.zeros((rows, nt))
    out[valid[:rows]] = values
    return out


def add_interface_damping(els, el_typ_i, K, C, M, gl_lookup, factor):
    """fn_add_interface_damping.m:30-52: C(gi, gi) += M(gi, gi) * level on
    every DOF of the fluid-solid interface nodes, level =
    min(sqrt(diag K / diag M)) / pi^2 * factor."""
    dK, dM = K.diagonal(), M.diagonal()
    with np.errstate(divide="ignore", invalid="ignore"):
        level = np.nanmin(np.sqrt(dK / dM)) / np.pi ** 2 * factor
    is_int = np.array([t == "ASI2D2" for t in el_typ_i])
    nd = np.asarray(els)[is_int]
    nd = nd[nd > 0]
    if nd.size == 0:
        return C
    gi = gl_lookup[nd - 1, :].ravel()
    gi = np.unique(gi[gi > 0]) - 1
    add = np.zeros(C.shape[0])
    add[gi] = dM[gi] * level
    return (C + sp.diags(add)).tocsr()


def build_matrices(mod, matls, opt):
    """fn_build_global_matrices_v5 for the 2D element types (CPE3, AC2D3,
    ASI2D2): K, C, M and gl_lookup, assembled on the GPU (``assemble_on_gpu``,
    the default) or by the vectorised host builder."""
    typ_names = list(mod["el_typ_i"])
    unknown = sorted(set(typ_names) - set(model.TYPE_CODES))
    if unknown:
        raise SolverError("element types %s are not supported by the GPU path's builder" % unknown)
    if opt.get("assemble_on_gpu", True):
        from .assembly import assemble_gpu
        K, C, M, gl = assemble_gpu(mod["nds"], mod["els"], mod["el_mat_i"], mod["el_abs_i"], typ_names, matls,
                                   dof_to_use=opt["dof_to_use"], damping_power_law=opt["damping_power_law"],
                                   max_damping=opt["max_damping"],
                                   max_stiffness_reduction=opt["max_stiffness_reduction"])
        if opt["interface_damping_factor"]:
            C = add_interface_damping(mod["els"], typ_names, K, C, M, gl, opt["interface_damping_factor"])
        return K, C, M, gl
    typ = np.array([model.TYPE_CODES[t] for t in typ_names])
    K, C, M, gl = model.assemble(np.asarray(mod["nds"], float), np.asarray(mod["els"], np.int64),
                                 np.asarray(mod["el_mat_i"], np.int64).ravel(),
                                 np.asarray(mod["el_abs_i"], float).ravel(), typ, matls,
                                 dof_to_use=opt["dof_to_use"], damping_power_law=opt["damping_power_law"],
                                 max_damping=opt["max_damping"],
                                 max_stiffness_reduction=opt["max_stiffness_reduction"])
    if opt["interface_damping_factor"]:
        C = add_interface_damping(mod["els"], typ_names, K, C, M, gl, opt["interface_damping_factor"])
    return K, C, M, gl


def _weighted(steps, values):
    """steps{1}.load.wts scales forces and displacements of every step
    (fn_BristolFE_v2.m:79-81, 92-94)."""
    if "wts" in steps[0]["load"]:
        return np.asarray(steps[0]["load"]["wts"], float).reshape(-1, 1) @ values
    return values


def fn_BristolFE_v2_gb300(mod, matls, steps, fe_options=None):
    """Drop-in for fn_BristolFE_v2 (code/fn_BristolFE_v2.m:1-157) returning
    (res, mats); with empty steps it returns the options with defaults
    (:32-37). res is a list with one dict per step holding dsps, dsp_gi,
    valid_mon_dsps, frcs, frc_gi, valid_appl_dsps, fld and fld_time as the
    reference's res{s} does."""
    opt = _set_default_fields(fe_options, DEFAULT_OPTIONS)
    if steps is None or (isinstance(steps, (list, tuple)) and len(steps) == 0):
        return opt
    opt = _set_default_fields(opt, DEFAULT_RUN_OPTIONS)
    mod = dict(mod)
    if "el_typ_i" not in mod:
        mod["el_typ_i"] = [matls[m - 1]["el_typ"] for m in np.asarray(mod["el_mat_i"]).ravel()]
    if "el_abs_i" not in mod:
        mod["el_abs_i"] = np.zeros(len(np.asarray(mod["el_mat_i"]).ravel()))
    K, C, M, gl = build_matrices(mod, matls, opt)
    mats = dict(K=K, C=C, M=M, gl_lookup=gl)
    if not isinstance(steps, (list, tuple)):
        steps = [steps]
    v5 = opt["dynamic_solver_version"] == "v5"
    mode = V5 if v5 else opt["solver_mode"]
    if not v5 and mode not in (VEL_CURRENT, VEL_LAST_HALF):
        raise SolverError("unknown solver_mode %r" % (mode,))
    precision = "double" if v5 else opt["solver_precision"]
    every = opt["field_output_every_n_frames"]
    ftype = opt["field_output_type"]

    # inputs of every step (fn_BristolFE_v2.m:73-107)
    jobs = []
    res = [dict() for _ in steps]
    for s, st in enumerate(steps):
        load = st["load"]
        if "time" not in load:
            jobs.append(None)
            continue
        r = res[s]
        t = np.asarray(load["time"], float).ravel()
        job = dict(t=t, frc_gi=np.zeros(0, np.int64), frcs=None, dsp_gi=np.zeros(0, np.int64), dsps=None)
        if "frcs" in load:
            job["frc_gi"], _, _, valid_f = nds_and_dfs_to_gi(load["frc_nds"], load["frc_dfs"], gl)
            frcs = _weighted(steps, np.atleast_2d(np.asarray(load["frcs"], float)))
            job["frcs"] = _mask_rows(frcs, valid_f) if frcs.shape[0] > 1 else frcs
        if "dsps" in load:
            job["dsp_gi"], _, _, r["valid_appl_dsps"] = nds_and_dfs_to_gi(load["dsp_nds"], load["dsp_dfs"], gl)
            dsps = _weighted(steps, np.atleast_2d(np.asarray(load["dsps"], float)))
            job["dsps"] = _mask_rows(dsps, r["valid_appl_dsps"]) if dsps.shape[0] > 1 else dsps
        mon = st.get("mon", {})
        job["has_mon"] = "nds" in mon
        if job["has_mon"]:
            job["hist_gi"], _, _, r["valid_mon_dsps"] = nds_and_dfs_to_gi(mon["nds"], mon["dfs"], gl)
        else:
            job["hist_gi"] = np.zeros(0, np.int64)
        jobs.append(job)

    if not any(j is not None for j in jobs):
        return res, mats
    frames = not np.isinf(every)
    fcode = field_type_code(ftype)
    plans = []
    # without step batching (or with one step) every run has one source, so
    # the plan skips the operator forms of batched runs
    one_source = not opt["batch_steps"] or sum(j is not None for j in jobs) == 1

    def plan_for(t):
        # one resident plan per time step size (steps normally share it)
        dt = t[1] - t[0]
        for p in plans:
            if abs(p.dt - dt) <= 1e-12 * abs(dt):
                return p
        plans.append(Plan(K, C, M, dt, mode, precision, gl, one_source=one_source))
        return plans[-1]

    field = FieldOutput(mod["nds"], mod["els"], gl, M, ftype) if frames and fcode is not None else None
    try:
        outs = _march(plan_for, jobs, v5, every, frames, field, opt["batch_steps"])
    finally:
        if field is not None:
            field.close()
        for p in plans:
            p.close()
    # results (fn_BristolFE_v2.m:125-147)
    for s, job in enumerate(jobs):
        if job is None:
            continue
        r = res[s]
        nt = job["t"].size
        h, fld, mf, r["fld_time"] = outs[s]
        if job["has_mon"]:
            r["dsps"] = _grow_rows(r["valid_mon_dsps"], h if h is not None else np.zeros((0, nt)), nt)
            r["dsp_gi"] = job["hist_gi"]
        else:
            r["dsps"], r["dsp_gi"] = None, None
        if job["dsps"] is not None:
            r["frcs"] = _grow_rows(r["valid_appl_dsps"], mf, nt)
            r["frc_gi"] = job["frc_gi"]        # the reference stores frc_gi here (:135)
        else:
            r["frcs"], r["frc_gi"] = None, None
        r["fld"] = fld if fld is not None else None
        if frames and fcode is None:
            r["fld"] = ftype                   # fn_get_field_output.m:61-62 returns the type string
    return res, mats


def _batchable(job, frames):
    return (job is not None and job["dsps"] is None and not frames and job["frc_gi"].size > 0
            and job["frcs"] is not None and job["frcs"].shape[1] >= job["t"].size)


def _march(plan_for, jobs, v5, every, frames, field, batch_steps):
    """Run every step; returns per step (hist, fld, force_output, fld_time)."""
    outs = [None] * len(jobs)
    pending = list(range(len(jobs)))
    if batch_steps and not v5:
        # group steps with the same time axis and monitors into one march
        groups = {}
        for s in pending:
            j = jobs[s]
            if not _batchable(j, frames):
                continue
            rows = j["frcs"].shape[0]
            key = (j["t"].size, j["t"][0], j["t"][-1], tuple(j["hist_gi"].tolist()),
                   rows if rows > 1 else 1)
            groups.setdefault(key, []).append(s)
        for key, members in groups.items():
            if len(members) < 2:
                continue
            rows = key[-1]
            if rows > 1 and len({jobs[s]["frc_gi"].size for s in members}) != 1:
                continue
            t = jobs[members[0]]["t"]
            nt = t.size
            F = np.stack([np.atleast_2d(jobs[s]["frcs"])[:, :nt] for s in members], axis=2)
            hist = plan_for(t).run_batched(t, [jobs[s]["frc_gi"] for s in members], F, jobs[members[0]]["hist_gi"])
            for k, s in enumerate(members):
                h = hist[:, :, k] if jobs[s]["hist_gi"].size else None
                outs[s] = (h, None, None, None)
                pending.remove(s)
    for s in pending:
        j = jobs[s]
        if j is None:
            continue
        plan = plan_for(j["t"])
        if v5:
            h, fld, mf, ft = plan.run_v5(j["t"], j["frc_gi"], j["frcs"], j["dsp_gi"], j["dsps"],
                                         j["hist_gi"], every)
            if fld is not None and field is not None:
                fld = field.apply(fld)
            elif fld is not None:
                fld = None
        else:
            if j["dsps"] is not None and j["dsp_gi"].size:
                raise SolverError("prescribed displacements are not supported by the v6 path "
                                  "(the reference reads an undefined u_previous, v6.m:191)")
            is_vel = field is None or field.field_output_type not in (
                "mean(u1)", "mean(u2)", "mean(u3)", "curl(u)", "div(u)")
            h, fld, ft = plan.run(j["t"], j["frc_gi"], j["frcs"], j["hist_gi"], every, is_vel, field=field)
            mf = None
            if field is None:
                fld = None
        if not j["hist_gi"].size:
            h = None
        outs[s] = (h, fld, mf, ft)
    return outs
