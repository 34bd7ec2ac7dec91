"""Element field output on the GPU: the mirror of fn_get_field_output
(code/internal/fn_get_field_output.m:1-135) over the native field kernels.

``FieldOutput`` uploads a model's mesh maps once; ``apply`` reduces frames
that are already on the host, and ``Plan.run(..., field=...)`` reduces each
frame on the device while the march produces it.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, ptr

MEAN_TYPES = ("mean(u1)", "mean(u2)", "mean(u3)", "mean(v1)", "mean(v2)", "mean(v3)")
DIV_TYPES = ("div(u)", "div(v)")
CURL_TYPES = ("curl(u)", "curl(v)")
RAW_TYPES = ("raw(u)", "raw(v)")


def field_type_code(field_output_type):
    """(BFE_FIELD_*, component) for a field_output_type string
    (fn_get_field_output.m:28-64); None for the raw types."""
    t = field_output_type
    if t in MEAN_TYPES:
        return _lib.BFE_FIELD_MEAN, int(t[6])                 # str2num(field_output_type(7))
    if t in DIV_TYPES:
        return _lib.BFE_FIELD_DIV, 0
    if t in CURL_TYPES:
        return _lib.BFE_FIELD_CURL, 0
    if t in RAW_TYPES:
        return None
    return _lib.BFE_FIELD_SQRT_KE, 0                          # 'otherwise %KE is the default'


class FieldOutput:
    """Device-resident mesh maps of one field_output_type for one model.

    nds: n_nodes x dims coordinates; els: n_el x cols 1-based nodes (0 =
    unused); gl_lookup: n_nodes x max_df 1-based global DOFs (0 = none);
    M: the global mass matrix (its diagonal, for sqrt(KE))."""

    def __init__(self, nds, els, gl_lookup, M, field_output_type="sqrt(KE)"):
        code = field_type_code(field_output_type)
        if code is None:
            raise ValueError("raw field output types have no element values")
        self.type, comp = code
        self.field_output_type = field_output_type
        self._lib = _lib.load()
        nds = np.asfortranarray(np.asarray(nds, float))
        els = np.asfortranarray(np.asarray(els, np.int64))
        gl = np.asfortranarray(np.asarray(gl_lookup, np.int64))
        self.n = int(M.shape[0])
        self.n_el = int(els.shape[0])
        m_diag = np.ascontiguousarray(M.diagonal(), dtype=float)
        self._keep = (nds, els, gl, m_diag)
        h = ctypes.c_void_p()
        st = self._lib.bfe_field_create(self.type, comp, self.n, gl.shape[0], nds.shape[1],
                                        ptr(nds, ctypes.c_double), gl.shape[1], ptr(gl, ctypes.c_int64),
                                        self.n_el, els.shape[1], ptr(els, ctypes.c_int64),
                                        ptr(m_diag, ctypes.c_double), ctypes.byref(h))
        check(st)
        self._h = h

    @property
    def handle(self):
        return self._h

    def apply(self, f_out):
        """Element values (n_el x n_frames) of frames f_out (n x n_frames)."""
        f = np.asfortranarray(np.asarray(f_out, float))
        if f.ndim == 1:
            f = f[:, None]
        if f.shape[0] != self.n:
            raise ValueError("frames have %d rows, the model has %d DOFs" % (f.shape[0], self.n))
        out = np.zeros((self.n_el, f.shape[1]), order="F")
        check(self._lib.bfe_field_apply(self._h, f.shape[1], ptr(f, ctypes.c_double),
                                        ptr(out, ctypes.c_double)))
        return out

    def close(self):
        if getattr(self, "_h", None):
            self._lib.bfe_field_destroy(self._h)
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


def fn_get_field_output_gb300(f_out, mod, mats, field_output_type="sqrt(KE)"):
    """Drop-in for fn_get_field_output(f_out, mod, mats, field_output_type):
    mod holds nds and els, mats holds M and gl_lookup. The raw types return
    the type string, as the reference does (fn_get_field_output.m:61-62)."""
    if field_type_code(field_output_type) is None:
        return field_output_type
    with FieldOutput(mod["nds"], mod["els"], mats["gl_lookup"], mats["M"], field_output_type) as fo:
        return fo.apply(f_out)
