"""ctypes binding of libbfe_gb300.so (the C ABI declared in include/bfe_gb300.h).

The library must exist: there is no CPU fallback. ``load()`` raises if the
shared object is missing or does not export every declared entry point.
"""
import ctypes
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libbfe_gb300.so")

BFE_OK = 0
BFE_ERR_ARG = 1
BFE_ERR_OOM = 2
BFE_ERR_CUDA = 3
BFE_ERR_NUMERIC = 4
BFE_ERR_UNSUPPORTED = 5
BFE_ERR_NO_DEVICE = 6
BFE_ERR_UNSTABLE = 7
BFE_ERR_TIMEOUT = 8
STATUS_NAMES = {0: "BFE_OK", 1: "BFE_ERR_ARG", 2: "BFE_ERR_OOM", 3: "BFE_ERR_CUDA",
                4: "BFE_ERR_NUMERIC", 5: "BFE_ERR_UNSUPPORTED", 6: "BFE_ERR_NO_DEVICE",
                7: "BFE_ERR_UNSTABLE", 8: "BFE_ERR_TIMEOUT"}

BFE_CSR = 0
BFE_CSC = 1
BFE_MODE_VEL_CURRENT = 0
BFE_MODE_VEL_LAST_HALF = 1
BFE_MODE_V5 = 2
BFE_EL_CPE3 = 0
BFE_EL_AC2D3 = 1
BFE_EL_ASI2D2 = 2
BFE_FIELD_SQRT_KE = 0
BFE_FIELD_MEAN = 1
BFE_FIELD_DIV = 2
BFE_FIELD_CURL = 3
BFE_PREC_DOUBLE = 0
BFE_PREC_SINGLE = 1
BFE_PLAN_ONE_SOURCE = 1

I64 = ctypes.c_int64
I32 = ctypes.c_int32
PD = ctypes.POINTER(ctypes.c_double)
PI64 = ctypes.POINTER(ctypes.c_int64)
PI32 = ctypes.POINTER(ctypes.c_int32)
VP = ctypes.c_void_p


class BfeSparse(ctypes.Structure):
    """bfe_sparse: a CSR or CSC view (0-based int64 indices, FP64 values)."""
    _fields_ = [("n_rows", I64), ("n_cols", I64), ("nnz", I64), ("format", I32),
                ("ptr", PI64), ("idx", PI64), ("val", PD)]


class BfeMesh2d(ctypes.Structure):
    """bfe_mesh2d: nodes, zero-padded 1-based element lists, materials,
    absorbing indices and element types (BFE_EL_*)."""
    _fields_ = [("n_nodes", I64), ("nds", PD), ("n_el", I64), ("el_cols", I32), ("els", PI64),
                ("el_mat", PI32), ("el_abs", PD), ("el_typ", PI32)]


class BfeMaterial(ctypes.Structure):
    """bfe_material: element type, density and the 6 x 6 (or scalar) D."""
    _fields_ = [("el_typ", I32), ("rho", ctypes.c_double), ("D", ctypes.c_double * 36)]


class BfeAssemblyOptions(ctypes.Structure):
    """bfe_assembly_options: DOFs in use (bit mask) and the absorber grading."""
    _fields_ = [("dof_mask", I32), ("damping_power_law", ctypes.c_double),
                ("max_damping", ctypes.c_double), ("max_stiffness_reduction", ctypes.c_double)]


class BfeStats(ctypes.Structure):
    """bfe_stats: counters of a plan's last run (bfe_plan_stats)."""
    _fields_ = [("step_launches", I64), ("aux_launches", I64), ("step_ms", ctypes.c_double),
                ("aux_ms", ctypes.c_double), ("n_dof", I64), ("nnz_stored", I64),
                ("nnz_padded", I64), ("n_interface", I64), ("n_direct_rows", I64),
                ("variant", I64), ("n_nodes", I64), ("n_groups", I64), ("adjoint_segments", I64),
                ("adjoint_kept", I64)]


SIGNATURES = {
    "bfe_plan_create": (I32, [ctypes.POINTER(BfeSparse), ctypes.POINTER(BfeSparse),
                              ctypes.POINTER(BfeSparse), ctypes.c_double, I32, I32,
                              PI64, PI32, ctypes.POINTER(VP)]),
    "bfe_plan_create_ex": (I32, [ctypes.POINTER(BfeSparse), ctypes.POINTER(BfeSparse),
                                 ctypes.POINTER(BfeSparse), ctypes.c_double, I32, I32,
                                 PI64, PI32, ctypes.c_uint32, ctypes.POINTER(VP)]),
    "bfe_plan_create_multi": (I32, [I32, ctypes.POINTER(BfeSparse), ctypes.POINTER(BfeSparse),
                                    ctypes.POINTER(BfeSparse), ctypes.c_double, I32, I32,
                                    ctypes.POINTER(PI64), ctypes.POINTER(PI32), PI64,
                                    ctypes.POINTER(VP)]),
    "bfe_plan_destroy": (I32, [VP]),
    "bfe_plan_ndof": (I32, [VP, PI64]),
    "bfe_run": (I32, [VP, I64, PD, I64, PI64, I64, PD, I64, PI64, I64, I32, PD, PD, PD]),
    "bfe_run_batched": (I32, [VP, I64, I64, PD, I64, PI64, I64, PD, I64, PI64, PD]),
    "bfe_assemble_2d": (I32, [ctypes.POINTER(BfeMesh2d), I32, ctypes.POINTER(BfeMaterial),
                              ctypes.POINTER(BfeAssemblyOptions), ctypes.POINTER(VP)]),
    "bfe_matrices_info": (I32, [VP, PI64, PI64, PI64, PI64, PI64, PI32]),
    "bfe_matrices_copy": (I32, [VP, I32, PI64, PI64, PD]),
    "bfe_matrices_gl_lookup": (I32, [VP, PI64]),
    "bfe_matrices_destroy": (I32, [VP]),
    "bfe_plan_create_assembled": (I32, [VP, ctypes.c_double, I32, I32, ctypes.POINTER(VP)]),
    "bfe_convolve": (I32, [I64, I64, PD, I64, PD, PD]),
    "bfe_fmc_gather": (I32, [I64, I64, I64, PD, I64, PI64, PI64, PI64, PD, I64, PD, PD]),
    "bfe_fmc_gather_device": (I32, [I64, I64, I64, VP, I64, PI64, PI64, PI64, PD, I64, PD, VP, VP]),
    "bfe_disps_to_forces": (I32, [ctypes.POINTER(BfeSparse), ctypes.POINTER(BfeSparse),
                                  ctypes.POINTER(BfeSparse), ctypes.c_double, I64, PD, PI32, I32, I32,
                                  PI64, PI64, PD]),
    "bfe_field_create": (I32, [I32, I32, I64, I64, I32, PD, I32, PI64, I64, I32, PI64, PD,
                               ctypes.POINTER(VP)]),
    "bfe_field_destroy": (I32, [VP]),
    "bfe_field_apply": (I32, [VP, I64, PD, PD]),
    "bfe_run_field": (I32, [VP, VP, I64, PD, I64, PI64, I64, PD, I64, PI64, I64, I32, PD, PD, PD]),
    "bfe_run_v5": (I32, [VP, I64, PD, I64, PI64, I64, PD, I64, PI64, I64, PD, I64, PI64, I64,
                         PD, PD, PD, PD]),
    "bfe_run_device": (I32, [VP, I64, I64, I64, I64, PI64, PI64, PI64, PD, I64, VP,
                             I64, PI64, VP, VP]),
    "bfe_adjoint_gradient": (I32, [VP, I64, I32, PI64, PD, PD, PD, I64, I64, PD, I64, PI64, I64, PD,
                                   I64, PI64, PD, I64, PD, PD, PD, PD]),
    "bfe_run_f64_noalloc": (I32, [I64, VP, VP, VP, VP, I64, I64, I64, VP, VP, VP, I64, VP, VP, VP]),
    "bfe_plan_set_timing": (I32, [VP, I32]),
    "bfe_plan_set_time_limit": (I32, [VP, ctypes.c_double]),
    "bfe_plan_stats": (I32, [VP, ctypes.POINTER(BfeStats)]),
    "bfe_last_error": (ctypes.c_char_p, []),
    "bfe_version": (I32, [PI32, PI32, PI32]),
}

_lib = None


class BfeError(RuntimeError):
    """A non-zero status returned across the C ABI.

    For BFE_ERR_UNSTABLE and BFE_ERR_TIMEOUT the run's outputs were still
    written; ``outputs`` then holds what the call would have returned."""

    def __init__(self, status, message, outputs=None):
        self.status = status
        self.outputs = outputs
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))


def load():
    """Load the native library (once). Raises if it is missing or incomplete."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libbfe_gb300.so not built (%s); run __graft_entry__.build()" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)          # AttributeError if not exported
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status, outputs=None):
    """Raise BfeError with bfe_last_error()'s message unless status is BFE_OK
    (``outputs`` is attached for the statuses after which they are valid)."""
    if status != BFE_OK:
        msg = load().bfe_last_error()
        keep = outputs if status in (BFE_ERR_UNSTABLE, BFE_ERR_TIMEOUT) else None
        raise BfeError(status, msg.decode() if msg else "", keep)


def ptr(a, ctype):
    """ctypes pointer to a contiguous numpy array (or NULL for None)."""
    if a is None:
        return ctypes.cast(None, ctypes.POINTER(ctype))
    return a.ctypes.data_as(ctypes.POINTER(ctype))
