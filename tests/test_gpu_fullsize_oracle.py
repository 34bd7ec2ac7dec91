"""The benchmarked sizes against the FP64 oracle (the C port of the
reference's v6 loop, oracle/c/cpu_march.c, with the exact interface P^-1).

C1 as configured: the coupled water/steel model (961,641 DOF, ASI2D2
interface chain of 1,200 edges, absorbers, void), one pressure source (the
array's centre element), 8,000 samples, the 64 element centres monitored and
a velocity field frame every 2,000 samples
(code/internal/fn_explicit_dynamic_solver_v6.m:180-218: history :196, frames
:200-208). The headline operator: the coupled model and the 32 steel
sub-domain models joined in one plan (6.31M DOF), sources 0 and 63 of the
64-source batched FP32 march and of the plain FP64 form, first 800 samples.

Tolerances (max-normalised, per model and per kind of DOF, since pressure and
displacement differ in units): FP64 1e-10, FP32 1e-4, for A-scans and
frames alike.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
TOL32 = 1e-4


def _group_err(a, b, groups):
    out = 0.0
    for g in groups:
        ref = np.abs(b[g]).max()
        assert ref > 0
        out = max(out, float(np.abs(a[g] - b[g]).max() / ref))
    return out


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


@pytest.fixture(scope="module")
def c1_case(bfe):
    """C1 model, signals, indices, and the oracle's A-scans and frames."""
    from bfe_gb300 import model
    from oracle import cpu_port
    m = model.coupled_water_steel()
    n_t, every = 8000, 2000
    t = np.arange(n_t) * m["dt"]
    sig = model.toneburst(t, 5e6, 5)
    fi = model.global_indices(m["gl"], m["src_nodes"][len(m["src_nodes"]) // 2], 4)
    hi = model.global_indices(m["gl"], m["mon_nodes"], 4)
    op = cpu_port.CpuOperator(m["K"], m["C"], m["M"], m["dt"])
    h0, f0, ft0 = op.march(t, fi - 1, sig[None, :], hi - 1, every, True, frames=True)
    from bfe_gb300.solver import dof_maps_from_lookup
    _, typ = dof_maps_from_lookup(m["gl"], m["K"].shape[0])
    groups = [np.nonzero(typ == 4)[0], np.nonzero(typ != 4)[0]]
    return dict(m=m, t=t, sig=sig, fi=fi, hi=hi, every=every, h0=h0, f0=f0, ft0=ft0, groups=groups)


@pytest.mark.parametrize("prec,tol", [("double", TOL64), ("single", TOL32)])
def test_c1_8000_samples_against_the_oracle(bfe, c1_case, prec, tol):
    c = c1_case
    m = c["m"]
    assert m["K"].shape[0] == 961641
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], bfe.VEL_CURRENT, prec,
                  m["gl"] if prec == "single" else None, one_source=True) as plan:
        h, f, ft = plan.run(c["t"], c["fi"], c["sig"], c["hi"], c["every"], True)
    assert np.abs(c["h0"]).max() > 0
    assert np.abs(h - c["h0"]).max() <= tol * np.abs(c["h0"]).max()
    assert f.shape == c["f0"].shape == (m["K"].shape[0], 4)
    assert np.array_equal(ft, c["ft0"])
    assert _group_err(f[:, 1:], c["f0"][:, 1:], c["groups"]) <= tol     # frame 0 precedes the pulse


@pytest.fixture(scope="module")
def headline(bfe):
    """The 33-model headline workload joined in one operator."""
    import bench
    from bfe_gb300 import model
    w = bench.workload(1.0)
    main, subs = bench.build_workload(w, 32)
    models = [main] + subs
    dt = min(m["dt"] for m in models)
    n_t = 800
    t = np.arange(n_t) * dt
    sig = model.toneburst(t, w["fc"], w["cycles"])
    return dict(models=models, dt=dt, t=t, sig=sig)


def _headline_indices(models, offs, R):
    from bfe_gb300 import model
    srcs = []
    for r in range(R):
        srcs.append(np.concatenate([model.global_indices(m["gl"], m["src_nodes"][r], 4 if k == 0 else 2) + offs[k]
                                    for k, m in enumerate(models)]))
    parts = [model.global_indices(m["gl"], m["mon_nodes"], 4 if k == 0 else 2) + offs[k]
             for k, m in enumerate(models)]
    groups, at = [], 0
    for p in parts:
        groups.append(np.arange(at, at + p.size))
        at += p.size
    return srcs, np.concatenate(parts), groups


def test_headline_sources_0_and_63_against_the_oracle(bfe, headline):
    import scipy.sparse as sp
    from oracle import cpu_port
    models, dt, t, sig = headline["models"], headline["dt"], headline["t"], headline["sig"]
    R = 64
    p32, offs = bfe.Plan.multi([(m["K"], m["C"], m["M"], m["gl"]) for m in models], dt, bfe.VEL_CURRENT, "single")
    srcs, mons, groups = _headline_indices(models, offs, R)
    assert p32.n == 6310411
    with p32:
        h32 = p32.run_batched(t, srcs, sig, mons)                 # (q, n_t, R)
    p64, _ = bfe.Plan.multi([(m["K"], m["C"], m["M"], None) for m in models], dt, bfe.VEL_CURRENT, "double")
    with p64:
        h64 = p64.run_batched(t, [srcs[0], srcs[R - 1]], sig, mons)
    op = cpu_port.CpuOperator(sp.block_diag([m["K"] for m in models], format="csr"),
                              sp.block_diag([m["C"] for m in models], format="csr"),
                              sp.block_diag([m["M"] for m in models], format="csr"), dt)
    for j, r in enumerate((0, R - 1)):
        h0 = op.march(t, srcs[r] - 1, sig[None, :], mons - 1)
        assert _group_err(h64[:, :, j], h0, groups) <= TOL64, r
        assert _group_err(h32[:, :, r], h0, groups) <= TOL32, r
