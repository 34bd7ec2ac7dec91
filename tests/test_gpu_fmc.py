"""GPU parity of the sub-domain / FMC post-processing (bfe_convolve,
bfe_fmc_gather, bfe_disps_to_forces) against the FP64 oracle. Tolerance:
max-normalised error <= 1e-12 (FP64; summation orders differ)."""
import numpy as np
import pytest

import modelgen
from oracle import subdomain
from oracle.solver import VEL_CURRENT, VEL_LAST_HALF

pytestmark = pytest.mark.gpu


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


@pytest.mark.parametrize("glen", [0.3, 0.5, 1.0, 3.0])
def test_convolve_matches_fft_convolution(bfe, glen):
    """Supports of 190 samples (direct sum) and 330 to 1,400 (the cuFFT route,
    g truncated to 2 n_t like fft(g, 2 n_t))."""
    rng = np.random.default_rng(3)
    n = 700
    f = rng.standard_normal((n, 6))
    g = rng.standard_normal(int(glen * n))
    g[: 20] = 0.0                                  # leading zeros (support search)
    ref = np.column_stack([subdomain.convolve(f[:, k], g) for k in range(f.shape[1])])
    assert _err(bfe.fn_convolve_gb300(f, g), ref) <= 1e-12


def test_convolve_with_a_recorded_history(bfe):
    """The sub-domain pipeline convolves recorded boundary histories (support
    = the whole record, subdoms/fn_run_subdomain_model.m:98-112): 16,384
    samples, 48 signals, against the oracle's FFT convolution."""
    rng = np.random.default_rng(11)
    n = 16384
    f = rng.standard_normal((n, 48))
    g = np.cumsum(rng.standard_normal(n)) * np.hanning(n)
    out = bfe.fn_convolve_gb300(f, g)
    for k in (0, 17, 47):
        ref = subdomain.convolve(f[:, k], g)
        assert _err(out[:, k], ref) <= 1e-12


def test_fmc_from_a_batched_run(bfe):
    m = modelgen.solid_plate(W=4e-3, H=2e-3, h=0.1e-3, dof_to_use=(1, 2))
    t, s = modelgen.pulse(400, m["dt"])
    nds = m["mod"]["nds"]
    top = np.nonzero(np.isclose(nds[:, 1], nds[:, 1].max()))[0]
    top = top[np.argsort(nds[top, 0])] + 1
    trans = [top[8 + 6 * k: 11 + 6 * k] for k in range(4)]            # 4 elements of 3 nodes
    mon = np.concatenate(trans)
    hi = modelgen.gi_of(m["gl"], mon, 2)
    srcs = [modelgen.gi_of(m["gl"], tr, 2) for tr in trans]
    impulse = np.zeros_like(s)
    impulse[0] = 1.0
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], VEL_CURRENT, "double") as plan:
        hist = plan.run_batched(t, srcs, impulse, hi)                  # (q, n_t, 4)
    tx = [a for a in range(4) for _ in range(4)]
    rx = [b for _ in range(4) for b in range(4)]
    wts = [None, np.array([0.25, 0.5, 0.25]), None, np.array([1.0, -1.0, 2.0])]
    dsps = [hist[:, :, r] for r in range(4)]
    ref = subdomain.parse_to_fmc(tx, rx, [mon] * 4, dsps, trans, wts, s)
    got = bfe.fn_parse_to_fmc_gb300(tx, rx, [mon] * 4, hist, trans, wts, s)
    assert got.shape == ref.shape == (400, 16)
    assert _err(got, ref) <= 1e-12
    raw = bfe.fn_parse_to_fmc_gb300(tx, rx, [mon] * 4, dsps, trans, wts, None)
    assert _err(raw, subdomain.parse_to_fmc(tx, rx, [mon] * 4, dsps, trans, wts, None)) <= 1e-12


@pytest.mark.parametrize("mode", [VEL_CURRENT, VEL_LAST_HALF])
@pytest.mark.parametrize("in_or_out", ["in", "out"])
def test_disps_to_forces_matches_oracle(bfe, mode, in_or_out):
    m = modelgen.solid_plate(W=3e-3, H=2e-3, h=0.1e-3, dof_to_use=(1, 2), abs_thick=0.6e-3)
    n = m["K"].shape[0]
    gl = m["gl"]
    x = m["mod"]["nds"][:, 0]
    node_of = np.zeros(n, np.int64)
    for d in range(gl.shape[1]):
        ok = gl[:, d] > 0
        node_of[gl[ok, d] - 1] = np.nonzero(ok)[0]
    lyrs = np.clip(np.floor(x[node_of] / 0.6e-3), 0, 4).astype(int)   # bands 0..4 across the plate
    rng = np.random.default_rng(4)
    t = np.arange(120) * m["dt"]
    disp = rng.standard_normal((n, 1)) * np.sin(2e6 * np.pi * t)[None, :] * 1e-9
    ref = subdomain.convert_disps_to_forces_v2(m["K"], m["C"], m["M"], m["dt"], disp, lyrs, in_or_out, mode)
    got = bfe.fn_convert_disps_to_forces_v2_gb300(m["K"], m["C"], m["M"], m["dt"], disp, lyrs, in_or_out, mode)
    for a, b in zip(got[1:], ref[1:]):
        assert np.array_equal(a, b)
    assert got[0].shape == ref[0].shape
    assert _err(got[0], ref[0]) <= 1e-12


@pytest.mark.parametrize("mode", [VEL_CURRENT, VEL_LAST_HALF])
@pytest.mark.parametrize("in_or_out", ["in", "out"])
def test_subdomain_forces_reproduce_the_field(bfe, mode, in_or_out):
    """The sub-domain principle end to end on the GPU: march a source, turn
    the displacement history into forces on layers 2 and 3
    (fn_convert_disps_to_forces_v2) with the frozen side zeroed, march those
    forces alone, and the field is reproduced on the kept side (layers 1-2
    for 'in', 3-4 for 'out') and zero on the frozen side. Layers are
    one-node-wide bands in x; the source sits on the frozen side."""
    m = modelgen.solid_plate(W=4e-3, H=2e-3, h=0.1e-3, dof_to_use=(1, 2), abs_thick=0.6e-3)
    n = m["K"].shape[0]
    gl = m["gl"]
    nds = m["mod"]["nds"]
    node_of = np.zeros(n, np.int64)
    for d in range(gl.shape[1]):
        ok = gl[:, d] > 0
        node_of[gl[ok, d] - 1] = np.nonzero(ok)[0]
    col = np.rint(nds[node_of, 0] / 0.1e-3).astype(int)          # node column of every DOF
    lyrs = np.select([col < 17, col == 17, col == 18], [4, 3, 2], 1)
    top = np.nonzero(np.isclose(nds[:, 1], nds[:, 1].max()))[0]
    src_x = 0.9e-3 if in_or_out == "in" else 3.0e-3               # frozen side
    src = top[np.argmin(np.abs(nds[top, 0] - src_x))] + 1
    fi = modelgen.gi_of(gl, [src], 2)
    nt = 260
    t, s = modelgen.pulse(nt, m["dt"])
    every = np.arange(1, n + 1)
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], mode, "double") as plan:
        U, _, _ = plan.run(t, fi, s, every)                          # all DOFs, n x n_t
        F, fset, _, _ = bfe.fn_convert_disps_to_forces_v2_gb300(m["K"], m["C"], m["M"], m["dt"], U, lyrs,
                                                                 in_or_out, mode)
        V, _, _ = plan.run(t, np.nonzero(fset)[0] + 1, F, every)
    kept = (lyrs <= 2) if in_or_out == "in" else (lyrs >= 3)
    scale = np.abs(U).max()
    assert np.abs(U[kept]).max() > 1e-3 * scale                      # the wave reaches the kept side
    assert np.abs(V[kept] - U[kept]).max() <= 1e-9 * scale
    assert np.abs(V[~kept]).max() <= 1e-9 * scale
