"""The MATLAB-side binding (bristolfe-v2_gb300/matlab/): the MEX gateways
compile (C99, -Wall -Wextra as errors) against include/bfe_gb300.h and a
stand-in mex.h, so every call into the C ABI matches the declared
signatures; the .m wrappers parse, and the v6 wrapper, run by the MATLAB
interpreter of tests/golden/mlab.py with its gateway bfe_mex stood in by the
oracle, reproduces the reference's own v6 results and rejects what the
reference rejects. MATLAB itself is not needed; nothing is linked."""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

import reference_golden as rg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MATLAB_DIR = os.path.join(ROOT, "bristolfe-v2_gb300", "matlab")
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
import mlab  # noqa: E402


@pytest.mark.parametrize("src", ["bfe_mex.c", "bfe_mex_v5.c"])
def test_gateway_compiles_against_the_abi(src):
    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-Wno-unused-parameter",
                        "-Wno-unused-function", "-fsyntax-only", "-I", os.path.join(ROOT, "tests", "mexstub"),
                        "-I", os.path.join(ROOT, "include"), os.path.join(MATLAB_DIR, src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_gateways_call_the_entry_points():
    v6 = open(os.path.join(MATLAB_DIR, "bfe_mex.c")).read()
    v5 = open(os.path.join(MATLAB_DIR, "bfe_mex_v5.c")).read()
    common = open(os.path.join(MATLAB_DIR, "bfe_mex_common.h")).read()
    assert "bfe_run(" in v6 and "mxSINGLE_CLASS" in common and "bfe_plan_create_ex" in common
    assert "bfe_run_v5(" in v5 and "BFE_MODE_V5" in v5


@pytest.mark.parametrize("name", ["fn_explicit_dynamic_solver_gb300", "fn_explicit_dynamic_solver_v5_gb300"])
def test_wrappers_parse(name):
    src = open(os.path.join(MATLAB_DIR, name + ".m")).read()
    funcs, order = mlab.Parser(mlab.lex(src)).parse_file()
    assert order[0] == name
    assert funcs[name][2][-1] == "varargin"                     # v6/v5 argument lists
    assert len(funcs[name][2]) == 11 and len(funcs[name][3]) == 4


def _oracle_gateway(calls):
    """bfe_mex stood in by the oracle: the gateway's 12 arguments in, its 3
    outputs out (1-based indices, the class of solver_precision)."""
    from oracle import solver as osolver

    def gateway(ip, a, n):
        K, C, M, time, fi, F, hi, every, is_vel, mode, prec, gl = a
        calls.append(str(prec))
        ftype = "KE" if mlab.scalar(is_vel) else "raw(u)"
        every = float(mlab.scalar(every))
        h, f, _, ft = osolver.explicit_dynamic_solver_v6(
            K.tocsr(), C.tocsr(), M.tocsr(), np.ravel(time), np.ravel(fi).astype(np.int64), np.asarray(F),
            [], [], np.ravel(hi).astype(np.int64), every, 0, ftype, str(mode))
        dt = np.float32 if str(prec).lower() == "single" else np.float64
        h = np.zeros((0, np.size(time))) if h is None else h
        f = np.zeros((0, 0)) if f is None else f
        ft = np.zeros((1, 0)) if ft is None else np.atleast_2d(ft)
        return [h.astype(dt), f.astype(dt), ft]
    return gateway


def test_v6_wrapper_run_by_the_interpreter_matches_the_reference():
    mod, matls, steps, opts, mats, gold = rg.case("coupled_lh")
    gl = mats["gl_lookup"]
    st = steps[0]
    fi = gl[st["load"]["frc_nds"] - 1, st["load"]["frc_dfs"] - 1].astype(float)
    hi_all = gl[st["mon"]["nds"] - 1, st["mon"]["dfs"] - 1]
    hi = hi_all[hi_all > 0].astype(float)
    calls = []
    ip = mlab.Interp([MATLAB_DIR], stubs={"bfe_mex": _oracle_gateway(calls)})
    args = [mats["K"], mats["C"], mats["M"], st["load"]["time"].reshape(1, -1), fi.reshape(-1, 1),
            st["load"]["frcs"], np.zeros((0, 0)), np.zeros((0, 0)), hi.reshape(-1, 1),
            opts["field_output_every_n_frames"], 1.0, opts["field_output_type"], opts["solver_mode"]]
    for prec in ("double", "single"):
        h, f, frc, ft = mlab.run(ip, "fn_explicit_dynamic_solver_gb300", args + [prec], 4)
        assert calls[-1] == prec
        assert h.dtype == (np.float32 if prec == "single" else np.float64)
        g = gold[0]["dsps"][np.nonzero(np.ravel(gold[0]["valid_mon_dsps"]))[0]]
        dfs = st["mon"]["dfs"][hi_all > 0]
        for rows in (dfs == 4, dfs != 4):
            tol = 1e-10 if prec == "double" else 1e-6
            assert np.abs(h[rows] - g[rows]).max() <= tol * np.abs(g[rows]).max()
        assert np.array_equal(np.ravel(ft), np.ravel(gold[0]["fld_time"]))
        assert mlab.numel(frc) == 0
    # no monitors and no frames: empty outputs, as v6.m:95-118
    h, f, frc, ft = mlab.run(ip, "fn_explicit_dynamic_solver_gb300",
                             args[:8] + [np.zeros((0, 0)), np.inf] + args[10:] + ["double"], 4)
    assert mlab.numel(h) == 0 and mlab.numel(f) == 0 and mlab.numel(ft) == 0
    # the reference's default solver_mode spelling matches neither of its cases
    with pytest.raises(mlab.MatlabError, match="solver_mode"):
        mlab.run(ip, "fn_explicit_dynamic_solver_gb300", args[:12], 4)
    # prescribed displacements are rejected (v6.m:191 reads an undefined variable)
    with pytest.raises(mlab.MatlabError, match="prescribed"):
        mlab.run(ip, "fn_explicit_dynamic_solver_gb300",
                 args[:6] + [np.array([[1.0]]), np.ones((1, args[3].size))] + args[8:] + ["double"], 4)
