"""Generate golden element-matrix vectors from the reference's own element code.

The reference's element routines ``code/internal/elements/fn_el_CPE3.m``,
``fn_el_AC2D3.m`` and ``fn_el_ASI2D2.m`` are machine-generated MATLAB files
whose bodies are element-wise arithmetic statements of the form
``el_K(:, i, j) = <expr>;`` over the per-element node coordinates
``nds_<node>_<dim>``, the material matrix ``D`` and density ``rho``. No MATLAB
exists here, so this script evaluates those statements directly: each
right-hand side is rewritten token-for-token into NumPy syntax
(``.*`` -> ``*``, ``./`` -> ``/``, ``.^`` -> ``**``, ``D(i, j)`` ->
``D[i-1, j-1]``) and evaluated on fixed inputs. The resulting arrays are the
reference's own numbers for those inputs and are stored in
``elements_golden.npz`` for the CPU tests, which compare the oracle's
independently derived element routines against them.

Run with the reference checkout's root as the first argument (or in the
environment variable REFERENCE_ROOT); the tests read only the stored fixture.
"""
import os
import re
import sys

import numpy as np

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("REFERENCE_ROOT", "")
ELDIR = os.path.join(REF, "code", "internal", "elements")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "elements_golden.npz")

_STMT = re.compile(r"^(J|el_K|el_C|el_M)\(:, (\d+), (\d+)\) = (.*);\s*$")


def _to_numpy(expr):
    e = expr.replace(".*", "*").replace("./", "/").replace(".^", "**")
    e = re.sub(r"\bD\((\d+), (\d+)\)", lambda m: f"D[{int(m.group(1)) - 1}, {int(m.group(2)) - 1}]", e)
    if "^" in e.replace("**", ""):
        raise ValueError("unsupported operator in: " + expr)
    return e


def evaluate_element_file(name, nds, els, D, rho):
    """Evaluate fn_el_<name>.m's statements for all elements (all DOFs)."""
    path = os.path.join(ELDIR, f"fn_el_{name}.m")
    with open(path) as f:
        lines = f.readlines()
    stmts = []
    ndf = 0
    for ln in lines:
        m = _STMT.match(ln.strip())
        if m:
            stmts.append((m.group(1), int(m.group(2)), int(m.group(3)), _to_numpy(m.group(4))))
        mz = re.match(r"^el_K = zeros\(size\(els, 1\), (\d+), (\d+)\);", ln.strip())
        if mz:
            ndf = int(mz.group(1))
    nel = els.shape[0]
    env = {"D": D, "rho": rho, "np": np}
    n_nodes_per_el = els.shape[1]
    for a in range(n_nodes_per_el):
        for d in range(nds.shape[1]):
            env[f"nds_{a + 1}_{d + 1}"] = nds[els[:, a] - 1, d]
    out = {k: np.zeros((nel, ndf, ndf)) for k in ("el_K", "el_C", "el_M")}
    for tgt, i, j, e in stmts:
        val = eval(e, {"__builtins__": {}}, env)
        if tgt == "J":
            env["J"] = np.broadcast_to(val, (nel,)).astype(float)
        else:
            out[tgt][:, i - 1, j - 1] = val
    return out["el_K"], out["el_C"], out["el_M"]


def main():
    if not os.path.isdir(ELDIR):
        print("reference element directory not found:", ELDIR)
        sys.exit(1)
    rng = np.random.default_rng(20240111)
    res = {}
    # CPE3 - random well-shaped triangles (both orientations) and the
    # builder's own unit triangle; random symmetric 6x6 D (el_sym_CPE3.m:91-96)
    nds = np.vstack([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0],
                     rng.uniform(-1e-3, 1e-3, size=(30, 2))])
    els = np.vstack([[1, 2, 3], [1, 3, 2],
                     np.arange(4, 34).reshape(10, 3)])
    A = rng.uniform(0.1, 1.0, size=(6, 6)) * 1e11
    D6 = A + A.T
    rho = 7850.5
    K, C, M = evaluate_element_file("CPE3", nds, els, D6, rho)
    res.update(cpe3_nds=nds, cpe3_els=els, cpe3_D=D6, cpe3_rho=rho, cpe3_K=K, cpe3_C=C, cpe3_M=M)
    # AC2D3 - scalar bulk modulus
    bulk = 2.25e9
    rho_w = 1000.0
    K, C, M = evaluate_element_file("AC2D3", nds, els, np.array(bulk), rho_w)
    res.update(ac2d3_bulk=bulk, ac2d3_rho=rho_w, ac2d3_K=K, ac2d3_C=C, ac2d3_M=M)
    # ASI2D2 - line elements at assorted angles (el_sym_ASI2D2.m:325)
    ang = np.deg2rad(np.array([0.0, 30.0, 90.0, 135.0, 200.0, 333.0]))
    L = np.array([1.0, 1.0, 2e-4, 5e-5, 3e-3, 1e-4])
    p1 = rng.uniform(-1e-3, 1e-3, size=(6, 2))
    p2 = p1 + L[:, None] * np.column_stack([np.cos(ang), np.sin(ang)])
    nds_i = np.empty((12, 2))
    nds_i[0::2] = p1
    nds_i[1::2] = p2
    els_i = np.arange(1, 13).reshape(6, 2)
    K, C, M = evaluate_element_file("ASI2D2", nds_i, els_i, np.zeros((6, 6)), 0.0)
    res.update(asi2d2_nds=nds_i, asi2d2_els=els_i, asi2d2_K=K, asi2d2_C=C, asi2d2_M=M)
    np.savez_compressed(OUT, **res)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
