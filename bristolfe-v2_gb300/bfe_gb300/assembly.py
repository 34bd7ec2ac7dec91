"""Global assembly on the GPU: the mirror of fn_build_global_matrices_v5
(code/internal/fn_build_global_matrices_v5.m:66-164) over the native
``bfe_assemble_2d`` kernels, for CPE3, AC2D3 and ASI2D2 meshes.

``DeviceMatrices`` keeps K, C and M on the device (``plan()`` builds a time
stepping plan from them); ``assemble_gpu`` returns them as SciPy CSR
matrices with the reference's gl_lookup.
"""
import ctypes

import numpy as np
import scipy.sparse as sp

from . import _lib
from ._lib import check, ptr
from .solver import Plan

TYPE_CODES = {"CPE3": _lib.BFE_EL_CPE3, "AC2D3": _lib.BFE_EL_AC2D3, "ASI2D2": _lib.BFE_EL_ASI2D2}


def _material(m):
    mat = _lib.BfeMaterial()
    mat.el_typ = TYPE_CODES.get(m.get("el_typ", "CPE3"), 0)
    mat.rho = float(m["rho"])
    D = np.asarray(m["D"], float)
    if D.ndim == 0 or D.size == 1:
        mat.D[0] = float(D)                                   # bulk modulus (fluid)
    else:
        flat = np.asfortranarray(D.reshape(6, 6)).ravel(order="F")
        for k in range(36):
            mat.D[k] = flat[k]
    return mat


class DeviceMatrices:
    """K, C, M and gl_lookup assembled on the current CUDA device."""

    def __init__(self, nds, els, el_mat, el_abs, el_typ, matls, dof_to_use=None, damping_power_law=3,
                 max_damping=3.1415e7, max_stiffness_reduction=0.01):
        self._lib = _lib.load()
        nds = np.asfortranarray(np.asarray(nds, float)[:, :2])
        els = np.asfortranarray(np.asarray(els, np.int64))
        el_mat = np.ascontiguousarray(np.asarray(el_mat, np.int32).ravel())
        el_abs = None if el_abs is None else np.ascontiguousarray(np.asarray(el_abs, float).ravel())
        codes = [TYPE_CODES[t] if isinstance(t, str) else int(t) for t in el_typ]
        el_typ = np.ascontiguousarray(np.asarray(codes, np.int32))
        mesh = _lib.BfeMesh2d(nds.shape[0], ptr(nds, ctypes.c_double), els.shape[0], els.shape[1],
                              ptr(els, ctypes.c_int64), ptr(el_mat, ctypes.c_int32),
                              ptr(el_abs, ctypes.c_double), ptr(el_typ, ctypes.c_int32))
        mats = (_lib.BfeMaterial * len(matls))(*[_material(m) for m in matls])
        mask = 0
        for d in (dof_to_use or []):
            mask |= 1 << (int(d) - 1)
        opt = _lib.BfeAssemblyOptions(mask, float(damping_power_law), float(max_damping),
                                      float(max_stiffness_reduction))
        h = ctypes.c_void_p()
        check(self._lib.bfe_assemble_2d(ctypes.byref(mesh), len(matls), mats, ctypes.byref(opt),
                                        ctypes.byref(h)))
        self._h = h
        n, nk, nc, nm, nn = (ctypes.c_int64() for _ in range(5))
        mdf = ctypes.c_int32()
        check(self._lib.bfe_matrices_info(h, ctypes.byref(n), ctypes.byref(nk), ctypes.byref(nc),
                                          ctypes.byref(nm), ctypes.byref(nn), ctypes.byref(mdf)))
        self.n, self.nnz, self.n_nodes, self.max_df = n.value, (nk.value, nc.value, nm.value), nn.value, mdf.value

    def matrix(self, which):
        """SciPy CSR copy of K (0), C (1) or M (2)."""
        nz = self.nnz[which]
        p = np.zeros(self.n + 1, np.int64)
        i = np.zeros(max(nz, 1), np.int64)
        v = np.zeros(max(nz, 1))
        check(self._lib.bfe_matrices_copy(self._h, which, ptr(p, ctypes.c_int64), ptr(i, ctypes.c_int64),
                                          ptr(v, ctypes.c_double)))
        return sp.csr_matrix((v[:nz], i[:nz], p), shape=(self.n, self.n))

    def gl_lookup(self):
        gl = np.zeros((self.n_nodes, self.max_df), np.int64, order="F")
        check(self._lib.bfe_matrices_gl_lookup(self._h, ptr(gl, ctypes.c_int64)))
        return np.ascontiguousarray(gl)

    def plan(self, dt, solver_mode, solver_precision="double"):
        """A Plan built from these matrices (node/DOF maps from the lookup)."""
        return Plan.from_handle_factory(
            lambda out, mode, prec: self._lib.bfe_plan_create_assembled(self._h, float(dt), mode, prec, out),
            self.n, dt, solver_mode, solver_precision)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.bfe_matrices_destroy(self._h)
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


def assemble_gpu(nds, els, el_mat, el_abs, el_typ, matls, dof_to_use=None, damping_power_law=3,
                 max_damping=3.1415e7, max_stiffness_reduction=0.01):
    """(K, C, M, gl_lookup) assembled on the GPU, as fn_build_global_matrices_v5."""
    with DeviceMatrices(nds, els, el_mat, el_abs, el_typ, matls, dof_to_use, damping_power_law,
                        max_damping, max_stiffness_reduction) as dm:
        return dm.matrix(0), dm.matrix(1), dm.matrix(2), dm.gl_lookup()
