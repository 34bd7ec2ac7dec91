"""The benchmark configurations at their full sizes.

C0 (the reference's CPU-runnable case) is compared with the FP64 oracle
sample by sample. The large configurations, too big for the oracle in test
time, are checked through properties that hold at any size: the march is
linear in the forcing (superposition, scaling) and a batched run equals the
separate runs of its sources. Tolerances: oracle parity 1e-10 (FP64) and
1e-4 (FP32) max-normalised; linearity and batched = single at the rounding
of the precision (1e-11 FP64, 1e-5 FP32, relative to the largest sample)."""
import numpy as np
import pytest

from oracle import solver as osolver

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


@pytest.fixture(scope="module")
def c1():
    from bfe_gb300 import model
    return model.coupled_water_steel()           # 60 x 30 mm at 0.05 mm, 961,641 DOF


@pytest.mark.parametrize("prec,tol", [("double", 1e-10), ("single", 1e-4)])
def test_c0_plate_full_config_against_the_oracle(bfe, prec, tol):
    """20 x 10 mm steel plate at 0.1 mm (40,602 DOF with dof_to_use [1 2]),
    2,000 samples, 16 top-surface monitors, a frame every 500 samples."""
    from bfe_gb300 import model
    m = model.steel_plate(W=20e-3, H=10e-3, h=0.1e-3, n_mon=16)
    assert m["K"].shape[0] == 40602
    t = np.arange(2000) * m["dt"]
    sig = model.toneburst(t, 5e6, 5)
    fi = model.global_indices(m["gl"], m["src_nodes"], 2)
    hi = model.global_indices(m["gl"], m["mon_nodes"], 2)
    h0, f0, _, ft0 = osolver.explicit_dynamic_solver_v6(m["K"], m["C"], m["M"], t, fi, sig, [], [], hi, 500, 0,
                                                        "KE", osolver.VEL_CURRENT)
    h1, f1, _, ft1 = bfe.fn_explicit_dynamic_solver_gb300(m["K"], m["C"], m["M"], t, fi, sig, [], [], hi, 500, 1,
                                                          "KE", osolver.VEL_CURRENT, prec, gl_lookup=m["gl"])
    assert _err(h1, h0) <= tol
    assert _err(f1, f0) <= tol and np.array_equal(ft1, ft0)


def test_c1_superposition_and_scaling_fp64(bfe, c1):
    """Two array elements fired together = the sum of firing each, and a
    scaled signal scales the A-scans (full coupled model, FP64, 600 samples)."""
    m = c1
    t = np.arange(600) * m["dt"]
    sig = np.zeros_like(t)
    sig[:400] = np.sin(2 * np.pi * 5e6 * t[:400]) * np.hanning(400)
    from bfe_gb300 import model
    a = model.global_indices(m["gl"], m["src_nodes"][10], 4)
    b = model.global_indices(m["gl"], m["src_nodes"][50], 4)
    mons = model.global_indices(m["gl"], m["mon_nodes"], 4)
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], bfe.VEL_CURRENT, "double") as plan:
        ha, _, _ = plan.run(t, a, sig, mons)
        hb, _, _ = plan.run(t, b, sig, mons)
        hab, _, _ = plan.run(t, np.concatenate([a, b]), sig, mons)
        h2, _, _ = plan.run(t, a, 2.5 * sig, mons)
    assert _err(hab, ha + hb) <= 1e-11
    assert _err(h2, 2.5 * ha) <= 1e-11


@pytest.mark.parametrize("prec,R,tol", [("double", 16, 1e-11), ("single", 64, 1e-5)])
def test_c1_batched_equals_single_runs(bfe, c1, prec, R, tol):
    """R array elements as R right-hand sides of one march (the group
    kernels) = the same sources marched one at a time (the one-source
    kernels), on the full coupled model."""
    m = c1
    from bfe_gb300 import model
    t = np.arange(400) * m["dt"]
    sig = model.toneburst(t, 5e6, 5)
    srcs = [model.global_indices(m["gl"], m["src_nodes"][k], 4) for k in range(R)]
    mons = model.global_indices(m["gl"], m["mon_nodes"], 4)
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], bfe.VEL_CURRENT, prec, m["gl"]) as plan:
        hb = plan.run_batched(t, srcs, sig, mons)
        for r in (0, R // 2, R - 1):
            h1, _, _ = plan.run(t, srcs[r], sig, mons)
            assert _err(hb[:, :, r], h1) <= tol, r


def test_c3_brick_linearity_fp32(bfe):
    """The 10 x 10 x 5 mm brick model (1,560,753 DOF): doubling the signal
    doubles the FP32 A-scans up to FP32 rounding."""
    from bfe_gb300 import model
    m = model.steel_block_3d()
    assert m["K"].shape[0] == 1560753
    t = np.arange(300) * m["dt"]
    sig = model.toneburst(t, 5e6, 5)
    fi = model.global_indices(m["gl"], m["src_nodes"][0], 3)
    hi = model.global_indices(m["gl"], m["mon_nodes"], 3)
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], bfe.VEL_CURRENT, "single", m["gl"]) as plan:
        h1, _, _ = plan.run(t, fi, sig, hi)
        h2, _, _ = plan.run(t, fi, 2.0 * sig, hi)
    assert np.abs(h1).max() > 0
    assert _err(h2, 2.0 * h1) <= 1e-5


def test_c1_fp32_within_1e4_of_fp64_over_8000_samples(bfe, c1):
    """C1 as configured: the coupled model (961,641 DOF, ASI2D2 interface,
    absorbers, void), one 5 MHz pressure source in the water (the array's
    centre element), 8,000 samples: the FP32 plan's A-scans at the 64
    element centres stay within 1e-4 (max-normalised) of the FP64 plan's,
    which the oracle pins at 1e-10 on the smaller cases."""
    m = c1
    from bfe_gb300 import model
    t = np.arange(8000) * m["dt"]
    sig = model.toneburst(t, 5e6, 5)
    fi = model.global_indices(m["gl"], m["src_nodes"][len(m["src_nodes"]) // 2], 4)
    hi = model.global_indices(m["gl"], m["mon_nodes"], 4)
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], bfe.VEL_CURRENT, "double", one_source=True) as p64:
        h64, _, _ = p64.run(t, fi, sig, hi)
    with bfe.Plan(m["K"], m["C"], m["M"], m["dt"], bfe.VEL_CURRENT, "single", m["gl"], one_source=True) as p32:
        h32, _, _ = p32.run(t, fi, sig, hi)
    assert np.abs(h64).max() > 0
    assert _err(h32, h64) <= 1e-4
