"""Loader of tests/golden/reference_runs.npz: golden vectors produced by
running the reference's own MATLAB code (fn_BristolFE_v2 and everything it
calls) in the interpreter of tests/golden/mlab.py, written by
tests/golden/make_reference_golden.py.

``case(name)`` returns (mod, matls, steps, fe_options, mats, res) with the
reference's inputs in the shapes the oracle's and the product's
fn_BristolFE_v2 mirrors take, and its outputs (mats: K, C, M as CSC,
gl_lookup; res: one dict per step)."""
import os

import numpy as np
import scipy.sparse as sp

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_runs.npz")
CASES = ("plate", "coupled_lh", "coupled_cur", "v5")
_G = None


def _g():
    global _G
    if _G is None:
        _G = np.load(PATH)
    return _G


def _group(prefix):
    """Entries under `prefix.` as a nested dict (sparse matrices rebuilt)."""
    g = _g()
    out = {}
    for k in g.files:
        if not k.startswith(prefix + "."):
            continue
        path = k[len(prefix) + 1:].split(".")
        d = out
        for p in path[:-1]:
            d = d.setdefault(p, {})
        d[path[-1]] = g[k]

    def fix(d):
        if isinstance(d, dict):
            if set(d) == {"data", "indices", "indptr", "shape"}:
                return sp.csc_matrix((d["data"], d["indices"], d["indptr"]), shape=tuple(d["shape"]))
            return {k: fix(v) for k, v in d.items()}
        if isinstance(d, np.ndarray) and d.dtype.kind == "U":
            return str(d) if d.ndim == 0 else [str(x) for x in d]
        return d
    return fix(out)


def _col(a):
    return np.asarray(a, float).ravel()


def case(name):
    g = _g()
    mod = _group(name + ".mod")
    mod = dict(nds=np.asarray(mod["nds"], float), els=np.asarray(mod["els"]).astype(np.int64),
               el_mat_i=_col(mod["el_mat_i"]).astype(np.int64), el_abs_i=_col(mod["el_abs_i"]),
               **({"el_typ_i": list(mod["el_typ_i"])} if "el_typ_i" in mod else {}))
    matls = []
    for k in range(int(g[name + ".n_matls"])):
        m = _group(name + ".matl%d" % k)
        D = np.asarray(m["D"], float)
        matls.append(dict(rho=float(m["rho"]), D=D if D.size > 1 else float(D.ravel()[0]), el_typ=m["el_typ"]))
    steps = []
    for k in range(int(g[name + ".n_steps"])):
        st = _group(name + ".step%d" % k)
        load = {}
        for key, v in st["load"].items():
            if key in ("frc_nds", "frc_dfs", "dsp_nds", "dsp_dfs"):
                load[key] = _col(v).astype(np.int64)
            elif key in ("time", "wts"):
                load[key] = _col(v)
            else:
                load[key] = np.atleast_2d(np.asarray(v, float))
        mon = {k2: _col(v).astype(np.int64) for k2, v in st.get("mon", {}).items()}
        steps.append(dict(load=load, mon=mon))
    opts = {}
    for key, v in _group(name + ".opts").items():
        if isinstance(v, str):
            opts[key] = v
        elif key == "dof_to_use":
            opts[key] = [int(x) for x in np.asarray(v).ravel()]
        else:
            x = float(np.asarray(v).ravel()[0])
            opts[key] = np.inf if np.isinf(x) else x
    mats = _group(name + ".mats")
    mats["gl_lookup"] = np.asarray(mats["gl_lookup"]).astype(np.int64)
    res = []
    for k in range(int(g[name + ".n_steps"])):
        r = _group(name + ".res%d" % k)
        res.append({key: (np.asarray(v) if not isinstance(v, str) else v) for key, v in r.items()})
    return mod, matls, steps, opts, mats, res


def groups(mod, steps):
    """Row groups for max-normalised comparisons, one scale per kind of
    quantity: per step, the history rows of pressure (DOF 4) and of
    displacement monitors; the element rows of each element type for field
    values."""
    hist = []
    for st in steps:
        dfs = np.asarray(st["mon"].get("dfs", []), np.int64)
        hist.append([np.nonzero(dfs == 4)[0], np.nonzero(dfs != 4)[0]])
    typ = np.asarray(mod.get("el_typ_i", ["CPE3"] * len(mod["el_mat_i"])))
    fld = [np.nonzero(typ == t)[0] for t in sorted(set(typ.tolist()))]
    return hist, fld
