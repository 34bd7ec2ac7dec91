"""The oracle (and the product's host-side assembly) against golden vectors
from the reference's own MATLAB code.

tests/golden/reference_runs.npz holds inputs and outputs of the reference's
fn_BristolFE_v2 (code/fn_BristolFE_v2.m) - global assembly with
fn_build_global_matrices_v5 and the element routines, interface damping,
fn_explicit_dynamic_solver_v6 in both solver modes and
fn_explicit_dynamic_solver_v5 with prescribed displacements,
fn_get_field_output - executed unmodified by the MATLAB interpreter in
tests/golden/mlab.py (tests/golden/make_reference_golden.py). This pins the
oracle's restatement to the reference at solver level: K, C, M to 1e-12,
gl_lookup and the index bookkeeping exactly, histories, frames and reaction
forces to 1e-10 (max-normalised). The GPU path is checked against the same
vectors in tests/test_gpu_reference_golden.py.
"""
import os
import sys

import numpy as np
import pytest

import reference_golden as rg
from oracle import entry, mesh

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import mlab  # noqa: E402

TOL = 1e-10


def _rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    assert a.shape == b.shape, (a.shape, b.shape)
    scale = np.abs(b).max() if b.size else 0.0
    return float(np.abs(a - b).max() / scale) if scale > 0 else float(np.abs(a - b).max() if a.size else 0.0)


def _empty(x):
    return x is None or (not isinstance(x, str) and np.asarray(x).size == 0)


def _group_rel(a, b, row_groups):
    """Largest max-normalised difference over groups of rows (each group
    scaled by its own largest reference value; groups that are all zero in
    the reference must be zero here too)."""
    out = 0.0
    for g in row_groups:
        g = g[g < b.shape[0]]
        if g.size:
            out = max(out, _rel(a[g], b[g]))
    return out


def check_res(res, gold, tol, hist_groups=None, fld_groups=None):
    """One step's results against the reference's res{s}: index bookkeeping
    exactly, histories (per DOF kind), reaction forces and element field
    values (per element type) within tol, max-normalised."""
    for key in ("valid_mon_dsps", "dsp_gi", "frc_gi", "valid_appl_dsps"):
        if key in gold and not _empty(gold[key]):
            assert np.array_equal(np.asarray(res[key]).astype(np.int64).ravel(),
                                  np.asarray(gold[key]).astype(np.int64).ravel()), key
    for key in ("dsps", "frcs", "fld"):
        g = gold.get(key)
        if _empty(g):
            assert _empty(res.get(key)), key
            continue
        g = np.atleast_2d(np.asarray(g, float))
        r = np.atleast_2d(np.asarray(res[key], float))
        assert r.shape == g.shape, (key, r.shape, g.shape)
        grp = {"dsps": hist_groups, "fld": fld_groups}.get(key) or [np.arange(g.shape[0])]
        err = _group_rel(r, g, grp)
        assert err <= tol, (key, err)
    if not _empty(gold.get("fld_time")):
        assert np.array_equal(np.asarray(res["fld_time"], float).ravel(), np.asarray(gold["fld_time"]).ravel())


@pytest.mark.parametrize("name", rg.CASES)
def test_oracle_entry_matches_reference_run(name):
    mod, matls, steps, opts, mats, gold = rg.case(name)
    res, m2 = entry.BristolFE_v2(mod, matls, steps, opts)
    for k in ("K", "C", "M"):
        assert m2[k].shape == mats[k].shape
        assert _rel(m2[k].toarray(), mats[k].toarray()) <= 1e-12, k
    assert np.array_equal(m2["gl_lookup"], mats["gl_lookup"])
    assert len(res) == len(gold)
    hist_g, fld_g = rg.groups(mod, steps)
    for r, g, hg in zip(res, gold, hist_g):
        check_res(r, g, TOL, hg, fld_g)


@pytest.mark.parametrize("name", rg.CASES)
def test_product_host_assembly_matches_reference_run(name):
    """bfe_gb300's host assembly (model.py, interface damping in entry.py)."""
    from bfe_gb300 import entry as pentry
    mod, matls, steps, opts, mats, gold = rg.case(name)
    opt = pentry._set_default_fields(dict(opts, assemble_on_gpu=False), pentry.DEFAULT_RUN_OPTIONS)
    if "el_typ_i" not in mod:
        mod = dict(mod, el_typ_i=[matls[m - 1]["el_typ"] for m in mod["el_mat_i"]])
    K, C, M, gl = pentry.build_matrices(mod, matls, opt)
    for k, A in (("K", K), ("C", C), ("M", M)):
        assert _rel(A.toarray(), mats[k].toarray()) <= 1e-12, k
    assert np.array_equal(gl, mats["gl_lookup"])


def test_oracle_meshes_match_reference_run():
    """The oracle's mesh, absorber and interface generators reproduce the
    models the reference's own generators built for the golden cases."""
    from oracle import signals
    mod, *_ = rg.case("plate")
    W, H, th = 2e-3, 1e-3, 0.3e-3
    m = mesh.rectangular_structured_mesh(np.array([[0, 0], [W, 0], [W, H], [0, H]]), 0.1e-3)
    m = mesh.add_absorbing_layer(m, np.array([[th, th], [W - th, th], [W - th, 2 * H], [th, 2 * H]]), th)
    assert np.abs(m["nds"] - mod["nds"]).max() <= 1e-18
    assert np.array_equal(m["els"], mod["els"])
    assert np.abs(np.ravel(m["el_abs_i"]) - mod["el_abs_i"]).max() <= 1e-12
    mod, matls, *_ = rg.case("coupled_lh")
    W, H, th = 2e-3, 2e-3, 0.4e-3
    steel = dict(rho=8000.0, D=signals.isotropic_stiffness_matrix(210e9, 0.3), el_typ="CPE3")
    water = dict(rho=1000.0, D=1500.0 ** 2 * 1000.0, el_typ="AC2D3")
    assert np.abs(steel["D"] - matls[0]["D"]).max() <= 1e-3
    m = mesh.rectangular_structured_mesh(np.array([[0, 0], [W, 0], [W, H], [0, H]]), 0.1e-3)
    m = mesh.set_els_inside_bdry_to_mat(m, np.array([[-1, H / 2], [W + 1, H / 2], [W + 1, H + 1], [-1, H + 1]]), 2)
    m = mesh.add_absorbing_layer(m, np.array([[th, th], [W - th, th], [W - th, 2 * H], [th, 2 * H]]), th)
    m["el_typ_i"] = [[steel, water][k - 1]["el_typ"] for k in np.ravel(m["el_mat_i"])]
    m = mesh.add_fluid_solid_interface_els(m, [steel, water])
    assert np.array_equal(m["els"], mod["els"])
    assert list(m["el_typ_i"]) == list(mod["el_typ_i"])
    assert np.array_equal(np.ravel(m["el_mat_i"]), mod["el_mat_i"])
    assert np.abs(np.ravel(m["el_abs_i"]) - mod["el_abs_i"]).max() <= 1e-12


# -- the interpreter itself: MATLAB semantics the golden runs rely on ----------

def _run(src, name="f", args=(), nout=1):
    ip = mlab.Interp([])
    funcs, order = mlab.Parser(mlab.lex(src)).parse_file()
    ip.files[name] = (funcs[order[0]], funcs)
    return mlab.run(ip, name, list(args), nout)


def test_interpreter_indexing_growth_and_deletion():
    src = """function [a, b, c, d, e] = f()
a = []; a(3) = 5;
b = zeros(2, 3); b(:, end + 1) = [7; 8];
c = 1:10; c([2 4]) = [];
d = reshape(1:24, 2, 3, 4); d = d(2, :, end);
x = [1 2; 3 4]; e = x(:)';
end
"""
    a, b, c, d, e = _run(src, nout=5)
    assert a.tolist() == [[0, 0, 5]]
    assert b.shape == (2, 4) and b[:, 3].tolist() == [7, 8]
    assert c.tolist() == [[1, 3, 5, 6, 7, 8, 9, 10]]
    assert d.tolist() == [[20, 22, 24]]
    assert e.tolist() == [[1, 3, 2, 4]]


def test_interpreter_structs_cells_and_builtins():
    src = """function [n, s, u, i, j, t] = f(m)
c = {m.name};
n = numel(c);
s = struct('a', 1); s.b.c = {2, 'x'}; s.b.c{3} = 4;
[u, i, j] = unique([3 1; 2 2; 3 1], 'rows');
t = sum(sparse([1 2 2], [1 1 1], [1 2 3], 2, 2));
end
"""
    n, s, u, i, j, t = _run(src, args=[[{"name": "p"}, {"name": "q"}]], nout=6)
    assert n.tolist() == [[2]]
    assert mlab.numel(s.a[0, 0]["b"].a[0, 0]["c"]) == 3
    assert u.tolist() == [[2, 2], [3, 1]] and j.ravel().tolist() == [2, 1, 2] and i.ravel().tolist() == [2, 1]
    assert t.tolist() == [[6, 0]]


def test_interpreter_rejects_unknown_functions():
    with pytest.raises(mlab.MatlabError):
        _run("function f()\nsystem('ls');\nend\n", nout=0)
