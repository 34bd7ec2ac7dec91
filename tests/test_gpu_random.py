"""Seeded random cases through the batched C ABI against the FP64 oracle:
model (solid plate with or without absorbers, DOFs 1-2 or 1-3; coupled
water/steel with or without a void), solver mode, precision, source count
(1 to 128, ragged forced-DOF lists), per-source signal rows, monitor set.
Each case draws its parameters from its own seed, so a failure names a
reproducible case. Tolerances as the parity tests: 1e-10 (FP64), 1e-4
(FP32), max-normalised."""
import numpy as np
import pytest

import modelgen
from oracle import solver as osolver

pytestmark = pytest.mark.gpu

TOL = {"double": 1e-10, "single": 1e-4}


def _err(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def bfe():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from bfe_gb300 import build
    build.build()
    import bfe_gb300
    bfe_gb300.load()
    return bfe_gb300


_MODELS = {}


def _model(kind):
    if kind not in _MODELS:
        if kind == "plate":
            _MODELS[kind] = modelgen.solid_plate(W=2.5e-3, H=1.2e-3, h=0.1e-3, dof_to_use=(1, 2))
        elif kind == "plate_abs_3dof":
            _MODELS[kind] = modelgen.solid_plate(W=2.5e-3, H=1.2e-3, h=0.1e-3, dof_to_use=(1, 2, 3),
                                                 abs_thick=0.4e-3)
        elif kind == "coupled":
            _MODELS[kind] = modelgen.coupled_model(W=2.4e-3, Hw=1.0e-3, Hs=1.0e-3, abs_thick=0.4e-3)
        else:
            _MODELS[kind] = modelgen.coupled_model(W=2.4e-3, Hw=1.0e-3, Hs=1.2e-3, abs_thick=0.4e-3, blob=True,
                                                   seed=4)
    return _MODELS[kind]


@pytest.mark.parametrize("seed", range(24))
def test_random_batched_case(bfe, seed):
    rng = np.random.default_rng(1000 + seed)
    kind = ["plate", "plate_abs_3dof", "coupled", "coupled_void"][rng.integers(4)]
    m = _model(kind)
    prec = ["double", "single"][seed % 2]                       # both precisions and modes
    mode = [osolver.VEL_CURRENT, osolver.VEL_LAST_HALF][(seed // 2) % 2]
    R = int(rng.choice([1, 2, 5, 16, 32, 64, 128]))
    nt = int(rng.integers(60, 180))
    t, s = modelgen.pulse(nt, m["dt"])
    gl = m["gl"]
    dofs = [d + 1 for d in range(gl.shape[1]) if (gl[:, d] > 0).any()]
    nodes = np.nonzero(gl.max(axis=1) > 0)[0] + 1
    srcs = []
    for r in range(R):
        d = int(rng.choice(dofs))                          # a DOF, then 1-3 nodes carrying it
        carriers = np.nonzero(gl[:, d - 1] > 0)[0] + 1
        pick = rng.choice(carriers, int(rng.integers(1, 4)), replace=False)
        srcs.append(modelgen.gi_of(gl, pick, d))
    p = max(x.size for x in srcs)
    F = s[None, :, None] * rng.uniform(0.5, 1.5, (p, 1, R))           # per-source signal rows
    q = int(rng.integers(1, 24))
    mon_nodes = rng.choice(nodes, q, replace=False)
    hi = np.concatenate([modelgen.gi_of(gl, mon_nodes, d) for d in dofs])
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], mode, prec, gl if rng.integers(2) else None) as plan:
        hb = plan.run_batched(t, srcs, F, hi)
    for r in sorted({0, R // 2, R - 1}):
        fr = F[: srcs[r].size, :, r]
        h0 = osolver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, srcs[r], fr, [], [], hi, np.inf, 0,
                                                "KE", mode)[0]
        assert _err(hb[:, :, r], h0) <= TOL[prec], (kind, prec, mode, R, r)
