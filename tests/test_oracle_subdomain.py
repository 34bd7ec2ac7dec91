"""Oracle checks of the sub-domain / FMC restatements (no GPU)."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import subdomain
from oracle.solver import VEL_CURRENT, VEL_LAST_HALF


def test_convolve_is_the_truncated_linear_convolution():
    rng = np.random.default_rng(0)
    f = rng.standard_normal(300)
    g = rng.standard_normal(120)
    h = subdomain.convolve(f, g)
    assert h.shape == f.shape
    assert np.abs(h - np.convolve(f, g)[:300]).max() <= 1e-12 * np.abs(h).max()


def test_convolve_wraps_like_the_fft_for_long_signals():
    # fft(g, 2 n) of a g longer than n brings its tail around the circle
    rng = np.random.default_rng(1)
    n = 50
    f = rng.standard_normal(n)
    g = rng.standard_normal(3 * n)
    h = subdomain.convolve(f, g)
    gt = g[: 2 * n]
    direct = np.array([sum(gt[tau] * (f[(t - tau) % (2 * n)] if (t - tau) % (2 * n) < n else 0.0)
                           for tau in range(2 * n)) for t in range(n)])
    assert np.abs(h - direct).max() <= 1e-12 * np.abs(h).max()


@pytest.mark.parametrize("mode", [VEL_CURRENT, VEL_LAST_HALF])
def test_disps_to_forces_of_a_rigid_layer_motion(mode):
    # a translation of every DOF gives K u = 0: the forces are m accn + C vel
    n = 12
    K = sp.diags([np.full(n - 1, -1.0), np.full(n, 2.0), np.full(n - 1, -1.0)], [-1, 0, 1]).tolil()
    K[0, 0] = K[-1, -1] = 1.0
    K = K.tocsr()
    C = sp.diags(np.linspace(0, 1, n)).tocsr()
    M = sp.diags(np.full(n, 3.0)).tocsr()
    lyrs = np.array([1, 1, 2, 2, 2, 3, 3, 3, 4, 4, 0, 0])
    t = np.arange(40) * 0.1
    disp = np.outer(np.ones(n), np.sin(t))
    f, fs, fi, fo = subdomain.convert_disps_to_forces_v2(K, C, M, 0.1, disp, lyrs, "out", mode)
    assert fs.sum() == 6 and fi.sum() == 3 and fo.sum() == 3
    # 'out' freezes layers 1 and 2: their displacements are zero, so rows of
    # layer 2 see K coupling to frozen neighbours
    assert f.shape == (6, 40) and np.isfinite(f).all()
    d = disp.copy()
    d[(lyrs == 1) | (lyrs == 2)] = 0
    tmp = np.hstack([np.zeros((n, 2)), d])
    acc = (tmp[:, 2:] - 2 * tmp[:, 1:-1] + tmp[:, :-2]) / 0.01
    row = np.nonzero(fs)[0][-1]
    v = (tmp[:, 2:] - tmp[:, :-2]) / 0.2 if mode == VEL_CURRENT else (tmp[:, 1:-1] - tmp[:, :-2]) / 0.1
    disp1 = np.hstack([np.zeros((n, 1)), d[:, :-1]])
    expect = 3.0 * acc[row] + C[row] @ v + K[row] @ disp1
    assert np.abs(f[-1] - expect).max() <= 1e-12 * np.abs(expect).max()


def test_parse_to_fmc_sums_or_weights_the_receiver_rows():
    rng = np.random.default_rng(2)
    mon = np.arange(10, 20)
    dsps = [rng.standard_normal((10, 30)) for _ in range(3)]
    trans = [np.array([10, 11]), np.array([15, 16, 17]), np.array([19])]
    wts = [None, np.array([0.5, 1.0, 2.0]), None]
    out = subdomain.parse_to_fmc([0, 1, 2], [1, 0, 2], [mon] * 3, dsps, trans, wts, None)
    assert np.allclose(out[:, 0], dsps[0][5:8].T @ np.array([0.5, 1.0, 2.0]))
    assert np.allclose(out[:, 1], dsps[1][0:2].sum(axis=0))
    assert np.allclose(out[:, 2], dsps[2][9])


@pytest.mark.parametrize("in_or_out", ["in", "out"])
def test_oracle_subdomain_forces_reproduce_the_field(in_or_out):
    """The sub-domain principle on the oracle: forces on layers 2 and 3 made
    from a march's displacement history (frozen side zeroed) reproduce that
    history on the kept side and nothing on the frozen side, to rounding."""
    import modelgen
    from oracle import solver as osolver
    m = modelgen.solid_plate(W=3e-3, H=1.5e-3, h=0.1e-3, dof_to_use=(1, 2), abs_thick=0.4e-3)
    n = m["K"].shape[0]
    gl = m["gl"]
    nds = m["mod"]["nds"]
    node_of = np.zeros(n, np.int64)
    for d in range(gl.shape[1]):
        ok = gl[:, d] > 0
        node_of[gl[ok, d] - 1] = np.nonzero(ok)[0]
    col = np.rint(nds[node_of, 0] / 0.1e-3).astype(int)
    lyrs = np.select([col < 12, col == 12, col == 13], [4, 3, 2], 1)
    top = np.nonzero(np.isclose(nds[:, 1], nds[:, 1].max()))[0]
    src = top[np.argmin(np.abs(nds[top, 0] - (0.6e-3 if in_or_out == "in" else 2.3e-3)))] + 1
    fi = np.array([gl[src - 1, 1]])
    t = np.arange(180) * m["dt"]
    s = np.sin(2 * np.pi * 5e6 * t) * np.hanning(t.size)
    every = np.arange(1, n + 1)
    U = osolver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, fi, s, [], [], every, np.inf, 0, "KE",
                                           osolver.VEL_CURRENT)[0]
    F, fset, _, _ = subdomain.convert_disps_to_forces_v2(m["K"], m["C"], m["M"], m["dt"], U, lyrs, in_or_out,
                                                         osolver.VEL_CURRENT)
    V = osolver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, np.nonzero(fset)[0] + 1, F, [], [], every,
                                           np.inf, 0, "KE", osolver.VEL_CURRENT)[0]
    kept = (lyrs <= 2) if in_or_out == "in" else (lyrs >= 3)
    scale = np.abs(U).max()
    assert np.abs(U[kept]).max() > 1e-3 * scale
    assert np.abs(V[kept] - U[kept]).max() <= 1e-12 * scale
    assert np.abs(V[~kept]).max() <= 1e-12 * scale
