"""Host-side mirror of the reference's time-marching call, backed by the C ABI.

``fn_explicit_dynamic_solver_gb300`` takes the arguments of
``fn_explicit_dynamic_solver_v6`` (code/internal/fn_explicit_dynamic_solver_v6.m:1-5)
with the same meaning - including 1-based global indices and MATLAB-shaped
arrays - and returns the same four outputs. All arithmetic runs in the native
library on the GPU; there is no CPU path here.
"""
import ctypes

import numpy as np
import scipy.sparse as sp

from . import _lib
from ._lib import BfeError, check, ptr

VEL_LAST_HALF = "vel at last half time step"     # v6.m:131
VEL_CURRENT = "vel at curent time step"          # v6.m:135 (sic)
DISP_FIELD_TYPES = ("mean(u1)", "mean(u2)", "mean(u3)", "curl(u)", "div(u)", "raw(u)")  # v6.m:64-69

V5 = "v5"                                        # fn_explicit_dynamic_solver_v5.m
_MODES = {VEL_CURRENT: _lib.BFE_MODE_VEL_CURRENT, VEL_LAST_HALF: _lib.BFE_MODE_VEL_LAST_HALF,
          V5: _lib.BFE_MODE_V5}


class SolverError(RuntimeError):
    """Raised where the reference solver raises (or fails) for the same input."""


def _mode_code(solver_mode):
    try:
        return _MODES[solver_mode]
    except KeyError:
        # v6.m:130-139 leaves A, B, D undefined for any other string
        raise SolverError("unknown solver_mode %r (accepted: %r, %r)"
                          % (solver_mode, VEL_CURRENT, VEL_LAST_HALF)) from None


def _precision_code(solver_precision):
    s = str(solver_precision).lower()
    if s == "single":
        return _lib.BFE_PREC_SINGLE
    if s == "double":
        return _lib.BFE_PREC_DOUBLE
    raise SolverError("solver_precision must be 'double' or 'single', got %r" % (solver_precision,))


def _csr_view(A, name):
    A = sp.csr_matrix(A)
    A.sum_duplicates()
    ptr_ = np.ascontiguousarray(A.indptr, dtype=np.int64)
    idx = np.ascontiguousarray(A.indices, dtype=np.int64)
    val = np.ascontiguousarray(A.data, dtype=np.float64)
    s = _lib.BfeSparse(A.shape[0], A.shape[1], val.size, _lib.BFE_CSR,
                       ptr(ptr_, ctypes.c_int64), ptr(idx, ctypes.c_int64), ptr(val, ctypes.c_double))
    return s, (ptr_, idx, val)


def dof_maps_from_lookup(gl_lookup, n):
    """(dof_node, dof_type) per global DOF from a reference gl_lookup matrix
    (rows = nodes, cols = DOF numbers, entries = 1-based global indices)."""
    gl = np.asarray(gl_lookup, dtype=np.int64)
    node = np.full(n, -1, np.int64)
    typ = np.zeros(n, np.int32)
    a, d = np.nonzero(gl > 0)
    g = gl[a, d] - 1
    if g.size and (g.max() >= n):
        raise SolverError("gl_lookup refers to DOFs beyond the matrix size")
    node[g] = a
    typ[g] = d + 1
    if np.any(node < 0):
        raise SolverError("gl_lookup does not cover every DOF")
    return node, typ


class Plan:
    """Device-resident time-stepping operator (one bfe_plan)."""

    def __init__(self, K, C, M, dt, solver_mode=VEL_CURRENT, solver_precision="double",
                 gl_lookup=None, one_source=False):
        """one_source: the plan serves one source per run (BFE_PLAN_ONE_SOURCE),
        so the operator forms of batched runs are not built."""
        lib = _lib.load()
        self._lib = lib
        self.mode = _mode_code(solver_mode)
        self.precision = _precision_code(solver_precision)
        self.dt = float(dt)
        n = K.shape[0]
        Ks, keepK = _csr_view(K, "K")
        Cs, keepC = _csr_view(C, "C")
        Ms, keepM = _csr_view(M, "M")
        node = typ = None
        if gl_lookup is not None:
            node, typ = dof_maps_from_lookup(gl_lookup, n)
        handle = ctypes.c_void_p()
        st = lib.bfe_plan_create_ex(ctypes.byref(Ks), ctypes.byref(Cs), ctypes.byref(Ms), self.dt,
                                    self.mode, self.precision, ptr(node, ctypes.c_int64),
                                    ptr(typ, ctypes.c_int32),
                                    _lib.BFE_PLAN_ONE_SOURCE if one_source else 0, ctypes.byref(handle))
        check(st)
        self._h = handle
        nn = ctypes.c_int64()
        check(lib.bfe_plan_ndof(self._h, ctypes.byref(nn)))
        self.n = nn.value

    @classmethod
    def multi(cls, models, dt, solver_mode=VEL_CURRENT, solver_precision="double"):
        """One plan over independent models joined block-diagonally.

        models: list of (K, C, M, gl_lookup or None). Returns (plan, offsets)
        where model k's 1-based DOF i is plan DOF offsets[k] + i."""
        lib = _lib.load()
        self = cls.__new__(cls)
        self._lib = lib
        self.mode = _mode_code(solver_mode)
        self.precision = _precision_code(solver_precision)
        self.dt = float(dt)
        nm = len(models)
        Ks = (_lib.BfeSparse * nm)()
        Cs = (_lib.BfeSparse * nm)()
        Ms = (_lib.BfeSparse * nm)()
        keep = []
        nodes = (_lib.PI64 * nm)()
        types = (_lib.PI32 * nm)()
        have_nodes = all(mdl[3] is not None for mdl in models)
        for k, (K, C, M, gl) in enumerate(models):
            for arr, A in ((Ks, K), (Cs, C), (Ms, M)):
                v, kp = _csr_view(A, "")
                arr[k] = v
                keep.append(kp)
            if have_nodes:
                nd, ty = dof_maps_from_lookup(gl, K.shape[0])
                keep.append((nd, ty))
                nodes[k] = ptr(nd, ctypes.c_int64)
                types[k] = ptr(ty, ctypes.c_int32)
        offs = np.zeros(nm + 1, np.int64)
        handle = ctypes.c_void_p()
        st = lib.bfe_plan_create_multi(nm, Ks, Cs, Ms, self.dt, self.mode, self.precision,
                                       nodes if have_nodes else None, types if have_nodes else None,
                                       ptr(offs, ctypes.c_int64), ctypes.byref(handle))
        check(st)
        self._h = handle
        nn = ctypes.c_int64()
        check(lib.bfe_plan_ndof(self._h, ctypes.byref(nn)))
        self.n = nn.value
        return self, offs

    @classmethod
    def from_handle_factory(cls, create, n, dt, solver_mode=VEL_CURRENT, solver_precision="double"):
        """A Plan whose handle comes from create(out, mode_code, precision_code)
        (e.g. bfe_plan_create_assembled)."""
        lib = _lib.load()
        self = cls.__new__(cls)
        self._lib = lib
        self.mode = _mode_code(solver_mode)
        self.precision = _precision_code(solver_precision)
        self.dt = float(dt)
        handle = ctypes.c_void_p()
        check(create(ctypes.byref(handle), self.mode, self.precision))
        self._h = handle
        nn = ctypes.c_int64()
        check(lib.bfe_plan_ndof(self._h, ctypes.byref(nn)))
        self.n = nn.value
        return self

    def set_timing(self, enable=True):
        """CUDA-event timing of every launch in later runs (see stats())."""
        check(self._lib.bfe_plan_set_timing(self._h, int(bool(enable))))

    def set_time_limit(self, seconds):
        """Wall-clock limit of later runs (0 = none): a run that passes it
        stops and raises BfeError(BFE_ERR_TIMEOUT) carrying the outputs
        computed so far."""
        check(self._lib.bfe_plan_set_time_limit(self._h, float(seconds)))

    def stats(self):
        """Counters of the last run as a dict (launches, device ms, nnz, ...)."""
        st = _lib.BfeStats()
        check(self._lib.bfe_plan_stats(self._h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in st._fields_}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.bfe_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def run(self, time, forcing_indices, forcing_functions, history_indices,
            field_output_every_n_frames=np.inf, field_is_vel=True, field=None):
        """One load step (1-based indices). Returns (hist q x n_t, fld or None, fld_time or None).

        With ``field`` (a FieldOutput of this model) each frame is reduced to
        element values on the device and fld is n_el x n_frames."""
        time = np.ascontiguousarray(np.asarray(time, float).ravel())
        nt = time.size
        fi = np.ascontiguousarray(np.asarray(forcing_indices, np.int64).ravel() - 1) \
            if forcing_indices is not None else np.zeros(0, np.int64)
        p = fi.size
        F = None
        rows = 0
        if p:
            F = np.atleast_2d(np.asarray(forcing_functions, float))
            if F.shape[1] < nt:
                raise SolverError("forcing_functions has fewer columns than time samples")
            F = np.asfortranarray(F[:, :nt])
            rows = F.shape[0]
        hi = np.ascontiguousarray(np.asarray(history_indices, np.int64).ravel() - 1) \
            if history_indices is not None else np.zeros(0, np.int64)
        q = hi.size
        hist = np.zeros((q, nt), order="F")
        every = 0 if np.isinf(field_output_every_n_frames) else int(field_output_every_n_frames)
        fld = fld_t = None
        if every > 0:
            nf = (nt + every - 1) // every
            fld = np.zeros((field.n_el if field is not None else self.n, nf), order="F")
            fld_t = np.zeros(nf)
        args = (nt, ptr(time, ctypes.c_double), p, ptr(fi, ctypes.c_int64),
                rows, ptr(F, ctypes.c_double), q, ptr(hi, ctypes.c_int64),
                every, int(bool(field_is_vel)), ptr(hist, ctypes.c_double),
                ptr(fld, ctypes.c_double), ptr(fld_t, ctypes.c_double))
        if field is not None:
            st = self._lib.bfe_run_field(self._h, field.handle, *args)
        else:
            st = self._lib.bfe_run(self._h, *args)
        check(st, (hist, fld, fld_t))
        return hist, fld, fld_t

    def run_v5(self, time, forcing_indices, forcing_functions, disp_indices, disp_functions,
               history_indices, field_output_every_n_frames=np.inf):
        """One load step of the v5 scheme (plan created with solver_mode V5),
        1-based indices, as fn_explicit_dynamic_solver_v5.m:60-188.

        Returns (hist q x n_t, fld n x n_frames or None, frc r x n_t or None,
        fld_time or None). Forcing shorter than time keeps its last column
        (v5.m:145-147); prescribed displacements need n_t columns."""
        time = np.ascontiguousarray(np.asarray(time, float).ravel())
        nt = time.size
        fi = np.ascontiguousarray(np.asarray(forcing_indices, np.int64).ravel() - 1) \
            if forcing_indices is not None else np.zeros(0, np.int64)
        p = fi.size
        F = None
        rows = 0
        if p:
            F = np.atleast_2d(np.asarray(forcing_functions, float))
            if F.shape[1] == 0:
                raise SolverError("forcing_functions is empty")
            if F.shape[1] < nt:
                F = np.hstack([F, np.repeat(F[:, -1:], nt - F.shape[1], axis=1)])
            F = np.asfortranarray(F[:, :nt])
            rows = F.shape[0]
        di = np.ascontiguousarray(np.asarray(disp_indices, np.int64).ravel() - 1) \
            if disp_indices is not None else np.zeros(0, np.int64)
        r = di.size
        D = None
        drows = 0
        frc = None
        if r:
            D = np.atleast_2d(np.asarray(disp_functions, float))
            if D.shape[1] < nt:
                raise SolverError("disp_functions has fewer columns than time samples")
            D = np.asfortranarray(D[:, :nt])
            drows = D.shape[0]
            frc = np.zeros((r, nt), order="F")
        hi = np.ascontiguousarray(np.asarray(history_indices, np.int64).ravel() - 1) \
            if history_indices is not None else np.zeros(0, np.int64)
        q = hi.size
        hist = np.zeros((q, nt), order="F")
        every = 0 if np.isinf(field_output_every_n_frames) else int(field_output_every_n_frames)
        fld = fld_t = None
        if every > 0:
            nf = (nt + every - 1) // every
            fld = np.zeros((self.n, nf), order="F")
            fld_t = np.zeros(nf)
        st = self._lib.bfe_run_v5(self._h, nt, ptr(time, ctypes.c_double), p, ptr(fi, ctypes.c_int64),
                                  rows, ptr(F, ctypes.c_double), r, ptr(di, ctypes.c_int64), drows,
                                  ptr(D, ctypes.c_double), q, ptr(hi, ctypes.c_int64), every,
                                  ptr(hist, ctypes.c_double), ptr(fld, ctypes.c_double),
                                  ptr(fld_t, ctypes.c_double), ptr(frc, ctypes.c_double))
        check(st, (hist, fld, frc, fld_t))
        return hist, fld, frc, fld_t

    def run_batched(self, time, forcing_indices_per_source, forcing_functions, history_indices):
        """R load steps sharing this operator as one multi-RHS march.

        forcing_indices_per_source: list of R 1-based index arrays (ragged ok);
        forcing_functions: (rows, n_t) shared by all sources or (rows, n_t, R),
        rows = 1 (broadcast) or the (common) number of forced DOFs.
        Returns hist of shape (q, n_t, R)."""
        time = np.ascontiguousarray(np.asarray(time, float).ravel())
        nt = time.size
        R = len(forcing_indices_per_source)
        p = max((len(np.ravel(x)) for x in forcing_indices_per_source), default=0)
        fi = np.full((p, R), -1, np.int64, order="F")
        for r, x in enumerate(forcing_indices_per_source):
            x = np.asarray(x, np.int64).ravel() - 1
            fi[: x.size, r] = x
        F = np.asarray(forcing_functions, float)
        if F.ndim == 1:
            F = F[None, :]
        if F.ndim == 2:
            F = np.repeat(F[:, :nt, None], R, axis=2)
        F = np.asfortranarray(F[:, :nt, :])
        rows = F.shape[0]
        hi = np.ascontiguousarray(np.asarray(history_indices, np.int64).ravel() - 1)
        q = hi.size
        hist = np.zeros((q, nt, R), order="F")
        st = self._lib.bfe_run_batched(self._h, R, nt, ptr(time, ctypes.c_double), p,
                                       ptr(fi, ctypes.c_int64), rows, ptr(F, ctypes.c_double),
                                       q, ptr(hi, ctypes.c_int64), ptr(hist, ctypes.c_double))
        check(st, hist)
        return hist

    def adjoint_gradient(self, element_data, time, forcing_indices_per_source, forcing_functions,
                         history_indices, observed, ckpt_every=0, return_history=False):
        """Misfit J and its gradients w.r.t. per-element stiffness scale and
        density (discrete adjoint). element_data = (ke, mh, ch, dof) with dof
        0-based global rows (n_el x ndf, -1 unused); indices 1-based; observed
        (q, n_t, R). ckpt_every = 0 keeps every forward state on the device
        when they fit (else checkpoints every ceil(sqrt(steps))); c > 0
        recomputes segments of c steps from checkpoints. Returns (J, g_stiff,
        g_rho[, hist])."""
        ke, mh, ch, dof = element_data
        ke = np.ascontiguousarray(ke, np.float64)
        mh = np.ascontiguousarray(mh, np.float64)
        ch = np.ascontiguousarray(ch, np.float64)
        dof = np.ascontiguousarray(dof, np.int64)
        n_el, ndf = dof.shape
        time = np.ascontiguousarray(np.asarray(time, float).ravel())
        nt = time.size
        R = len(forcing_indices_per_source)
        p = max(len(np.ravel(x)) for x in forcing_indices_per_source)
        fi = np.full((p, R), -1, np.int64, order="F")
        for r, x in enumerate(forcing_indices_per_source):
            x = np.asarray(x, np.int64).ravel() - 1
            fi[: x.size, r] = x
        F = np.asarray(forcing_functions, float)
        if F.ndim == 1:
            F = F[None, :]
        if F.ndim == 2:
            F = np.repeat(F[:, :nt, None], R, axis=2)
        F = np.asfortranarray(F[:, :nt, :])
        hi = np.ascontiguousarray(np.asarray(history_indices, np.int64).ravel() - 1)
        obs = np.asfortranarray(np.asarray(observed, float))
        J = ctypes.c_double()
        gs = np.zeros(n_el)
        gr = np.zeros(n_el)
        hist = np.zeros((hi.size, nt, R), order="F")
        st = self._lib.bfe_adjoint_gradient(
            self._h, n_el, ndf, ptr(dof, ctypes.c_int64), ptr(ke, ctypes.c_double),
            ptr(mh, ctypes.c_double), ptr(ch, ctypes.c_double), R, nt, ptr(time, ctypes.c_double),
            p, ptr(fi, ctypes.c_int64), F.shape[0], ptr(F, ctypes.c_double), hi.size,
            ptr(hi, ctypes.c_int64), ptr(obs, ctypes.c_double), int(ckpt_every), ctypes.byref(J),
            ptr(gs, ctypes.c_double), ptr(gr, ctypes.c_double), ptr(hist, ctypes.c_double))
        check(st)
        return (J.value, gs, gr, hist) if return_history else (J.value, gs, gr)

    def run_device(self, R, n_t, ti_start, frc_dof, frc_rhs, frc_sig, frc_w, d_sig, hist_idx,
                   d_hist, stream=0):
        """Device-resident march: d_sig / d_hist are torch CUDA tensors (FP64).

        frc_* are 0-based host arrays; d_hist must be zeroed, shape (R, n_t, q)
        in C order == q x n_t x R column-major."""
        frc_dof = np.ascontiguousarray(frc_dof, np.int64)
        frc_rhs = np.ascontiguousarray(frc_rhs, np.int64)
        frc_sig = np.ascontiguousarray(frc_sig, np.int64)
        frc_w = None if frc_w is None else np.ascontiguousarray(frc_w, np.float64)
        hist_idx = np.ascontiguousarray(hist_idx, np.int64)
        st = self._lib.bfe_run_device(
            self._h, int(R), int(n_t), int(ti_start), frc_dof.size, ptr(frc_dof, ctypes.c_int64),
            ptr(frc_rhs, ctypes.c_int64), ptr(frc_sig, ctypes.c_int64),
            ptr(frc_w, ctypes.c_double), int(d_sig.shape[-1]) if d_sig is not None else 0,
            ctypes.c_void_p(d_sig.data_ptr() if d_sig is not None else 0),
            hist_idx.size, ptr(hist_idx, ctypes.c_int64),
            ctypes.c_void_p(d_hist.data_ptr() if d_hist is not None else 0),
            ctypes.c_void_p(int(stream)))
        check(st)


def fn_explicit_dynamic_solver_gb300(K, C, M, time, forcing_indices, forcing_functions,
                                     disp_indices, disp_functions, history_indices,
                                     field_output_every_n_frames, use_gpu_if_present=1,
                                     field_output_type="KE", solver_mode=VEL_CURRENT,
                                     solver_precision="double", gl_lookup=None):
    """Drop-in for fn_explicit_dynamic_solver_v6 (same 14 arguments, 1-based
    indices). Returns (history_output, field_output, force_output,
    field_output_time); force_output is always None because prescribed
    displacements are rejected, as in the reference's v6 path (v6.m:191).

    ``gl_lookup`` (optional, the builder's node/DOF lookup) enables the
    translation-invariant FP32 stiffness product."""
    if K.shape[0] != K.shape[1]:
        raise SolverError("K must be square matrix")
    if C.shape[0] != C.shape[1]:
        raise SolverError("C must be square matrix")
    if M.shape[0] != M.shape[1]:
        raise SolverError("M must be square matrix")
    if disp_indices is not None and len(np.ravel(disp_indices)):
        raise SolverError("prescribed displacements are not supported by the v6 path "
                          "(the reference reads an undefined u_previous, v6.m:191)")
    if solver_mode not in (VEL_CURRENT, VEL_LAST_HALF):
        raise SolverError("unknown solver_mode %r (accepted: %r, %r)"
                          % (solver_mode, VEL_CURRENT, VEL_LAST_HALF))
    time = np.asarray(time, float).ravel()
    dt = time[1] - time[0]
    is_vel = field_output_type not in DISP_FIELD_TYPES
    # node information serves the FP32 difference form; an FP64 plan would
    # only use it for many-source kernels, which one load step never runs
    single = _precision_code(solver_precision) == _lib.BFE_PREC_SINGLE
    with Plan(K, C, M, dt, solver_mode, solver_precision, gl_lookup if single else None, one_source=True) as plan:
        hist, fld, fld_t = plan.run(time, forcing_indices, forcing_functions, history_indices,
                                    field_output_every_n_frames, is_vel)
    if history_indices is None or len(np.ravel(history_indices)) == 0:
        hist = None
    return hist, fld, None, fld_t


def fn_explicit_dynamic_solver_v5_gb300(K, C, M, time, forcing_indices, forcing_functions,
                                        disp_indices, disp_functions, history_indices,
                                        field_output_every_n_frames, use_gpu_if_present=1,
                                        solver_precision="double", gl_lookup=None):
    """Drop-in for fn_explicit_dynamic_solver_v5 (its 11 arguments, 1-based
    indices; v5.m:1-5). Returns (history_output, field_output, force_output,
    field_output_time); the field output is the velocity (v5.m:31,168-177).

    ``solver_precision`` and ``gl_lookup`` are extensions: the reference's v5
    is FP64 only."""
    n = K.shape[0]
    if K.shape[0] != K.shape[1]:
        raise SolverError("K must be square matrix")                          # v5.m:50-52
    if C.shape != (n, n):
        raise SolverError("C must be square matrix, same size as K")          # v5.m:53-55
    if M.shape != (n, n):
        raise SolverError("M must be square matrix, same size as K")          # v5.m:56-58
    time = np.asarray(time, float).ravel()
    dt = time[1] - time[0]
    single = _precision_code(solver_precision) == _lib.BFE_PREC_SINGLE
    with Plan(K, C, M, dt, V5, solver_precision, gl_lookup if single else None, one_source=True) as plan:
        hist, fld, frc, fld_t = plan.run_v5(time, forcing_indices, forcing_functions, disp_indices,
                                            disp_functions, history_indices,
                                            field_output_every_n_frames)
    if history_indices is None or len(np.ravel(history_indices)) == 0:
        hist = None
    return hist, fld, frc, fld_t
