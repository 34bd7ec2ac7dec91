"""C ABI checks that need no GPU: the library builds, loads, exports every
entry point declared in include/bfe_gb300.h, and rejects bad arguments on the
host before touching a device."""
import ctypes
import os
import re

import numpy as np
import pytest
import scipy.sparse as sp

import conftest

HEADER = os.path.join(conftest.ROOT, "include", "bfe_gb300.h")


def _lib():
    from bfe_gb300 import _lib as L
    from bfe_gb300 import build as B
    if not os.path.exists(L.LIB_PATH):
        B.build()
    return L, L.load()


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(bfe_\w+)\s*\(", src, flags=re.M)))


def test_header_declares_expected_entry_points():
    names = declared_functions()
    for n in ("bfe_plan_create", "bfe_plan_destroy", "bfe_run", "bfe_run_batched",
              "bfe_run_device", "bfe_last_error", "bfe_version", "bfe_plan_ndof"):
        assert n in names


def test_library_exports_every_declared_symbol():
    L, lib = _lib()
    for name in declared_functions():
        assert hasattr(lib, name), name
        assert name in L.SIGNATURES, "binding missing for " + name


def test_version():
    L, lib = _lib()
    a, b, c = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    assert lib.bfe_version(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)) == 0
    assert (a.value, b.value) >= (0, 1)


def _view(L, A):
    A = sp.csr_matrix(A)
    p = A.indptr.astype(np.int64); i = A.indices.astype(np.int64); v = A.data.astype(np.float64)
    s = L.BfeSparse(A.shape[0], A.shape[1], v.size, L.BFE_CSR, L.ptr(p, ctypes.c_int64),
                    L.ptr(i, ctypes.c_int64), L.ptr(v, ctypes.c_double))
    return s, (p, i, v)


def _create(L, lib, K, C, M, dt=1e-8, mode=0, prec=0):
    ks, k_ = _view(L, K); cs, c_ = _view(L, C); ms, m_ = _view(L, M)
    h = ctypes.c_void_p()
    st = lib.bfe_plan_create(ctypes.byref(ks), ctypes.byref(cs), ctypes.byref(ms), dt, mode, prec,
                             None, None, ctypes.byref(h))
    return st, h


def test_bad_arguments_are_rejected_on_host():
    L, lib = _lib()
    n = 4
    K = sp.identity(n) * 2.0
    M = sp.identity(n)
    C = sp.csr_matrix((n, n))
    st, _ = _create(L, lib, K, C, M, mode=7)
    assert st == L.BFE_ERR_ARG and b"solver_mode" in lib.bfe_last_error()
    st, _ = _create(L, lib, K, C, M, prec=3)
    assert st == L.BFE_ERR_ARG
    st, _ = _create(L, lib, K, C, M, dt=-1.0)
    assert st == L.BFE_ERR_ARG
    st, _ = _create(L, lib, sp.csr_matrix(np.ones((3, 4))), C, M)
    assert st == L.BFE_ERR_ARG
    Mz = sp.diags([1.0, 0.0, 1.0, 1.0])
    st, _ = _create(L, lib, K, C, Mz)
    assert st in (L.BFE_ERR_NUMERIC, L.BFE_ERR_NO_DEVICE)
    bad = sp.csr_matrix(np.diag([1.0, np.nan, 1.0, 1.0]))
    st, _ = _create(L, lib, bad, C, M)
    assert st == L.BFE_ERR_NUMERIC
    ks, k_ = _view(L, K); cs, c_ = _view(L, C); ms, m_ = _view(L, M)
    h = ctypes.c_void_p()
    st = lib.bfe_plan_create_ex(ctypes.byref(ks), ctypes.byref(cs), ctypes.byref(ms), 1e-8, 0, 0, None, None,
                                0x6, ctypes.byref(h))
    assert st == L.BFE_ERR_ARG and b"flags" in lib.bfe_last_error()


def test_null_plan_calls_fail_cleanly():
    L, lib = _lib()
    t = np.arange(4, dtype=float)
    st = lib.bfe_run(None, 4, L.ptr(t, ctypes.c_double), 0, None, 0, None, 0, None, 0, 1,
                     None, None, None)
    assert st == L.BFE_ERR_ARG
    assert lib.bfe_plan_destroy(None) == 0


def test_plan_create_without_gpu_reports_no_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L, lib = _lib()
    n = 4
    st, _ = _create(L, lib, sp.identity(n) * 2.0, sp.csr_matrix((n, n)), sp.identity(n))
    assert st == L.BFE_ERR_NO_DEVICE
    assert b"device" in lib.bfe_last_error()


def test_python_mirror_rejects_like_reference():
    from bfe_gb300 import solver as S
    n = 4
    K = sp.identity(n); C = sp.csr_matrix((n, n)); M = sp.identity(n)
    t = np.arange(5) * 1e-8
    with pytest.raises(S.SolverError):
        S.fn_explicit_dynamic_solver_gb300(K, C, M, t, [1], np.ones(5), [2], np.ones(5), [1],
                                           np.inf)
    with pytest.raises(S.SolverError):
        S._mode_code("vel at current time step")    # v6's own default spelling fails in v6
    with pytest.raises(S.SolverError):
        S._precision_code("half")
    assert S._precision_code("SINGLE") == 1


def test_dof_maps_from_lookup():
    from bfe_gb300 import solver as S
    gl = np.array([[1, 2, 0, 0], [3, 4, 0, 5], [0, 0, 0, 6]])
    node, typ = S.dof_maps_from_lookup(gl, 6)
    assert node.tolist() == [0, 0, 1, 1, 1, 2]
    assert typ.tolist() == [1, 2, 1, 2, 4, 4]


def test_assembly_argument_errors_are_caught_on_host():
    """bfe_assemble_2d validates the mesh before touching a device."""
    import bfe_gb300
    import modelgen
    m = modelgen.solid_plate(W=1e-3, H=1e-3, h=0.2e-3)
    mod = m["mod"]
    els = np.array(mod["els"]).copy()
    els[3, 1] = mod["nds"].shape[0] + 7
    with pytest.raises(bfe_gb300.BfeError, match="node out of range"):
        bfe_gb300.assemble_gpu(mod["nds"], els, mod["el_mat_i"], None, m["typ"], m["matls"])
    with pytest.raises(bfe_gb300.BfeError, match="material out of range"):
        bfe_gb300.assemble_gpu(mod["nds"], mod["els"], np.full(len(els), 5), None, m["typ"], m["matls"])
    bad = np.array(m["typ"], dtype=object)
    with pytest.raises(KeyError):
        bfe_gb300.assemble_gpu(mod["nds"], mod["els"], mod["el_mat_i"], None, ["HEX8"] * len(bad), m["matls"])


def test_postprocessing_argument_errors_are_caught_on_host():
    L, lib = _lib()
    h = np.zeros(4)
    assert lib.bfe_convolve(0, 1, None, 0, None, None) == L.BFE_ERR_ARG
    assert lib.bfe_convolve(4, 1, None, 1, None, L.ptr(h, ctypes.c_double)) == L.BFE_ERR_ARG
    assert lib.bfe_fmc_gather(0, 4, 1, None, 1, None, None, None, None, 0, None, None) == L.BFE_ERR_ARG
    n_force = ctypes.c_int64()
    assert lib.bfe_disps_to_forces(None, None, None, 1.0, 4, None, None, 0, 0, ctypes.byref(n_force),
                                   None, None) == L.BFE_ERR_ARG
    assert b"NULL" in lib.bfe_last_error()
