"""Host logic of the entry mirror (no GPU): options, index mapping, the
builder with interface damping against the oracle."""
import numpy as np

import modelgen
from oracle import assembly as oassembly
from oracle import entry as oentry


def test_options_only_call_returns_defaults():
    from bfe_gb300.entry import fn_BristolFE_v2_gb300
    opts = fn_BristolFE_v2_gb300({}, [], [], {"field_output_type": "mean(u1)"})
    assert opts["dynamic_solver_version"] == "v6"
    assert opts["global_matrix_builder_version"] == "v5"
    assert opts["solver_mode"] == "vel at curent time step"
    assert opts["field_output_type"] == "mean(u1)"
    assert opts["use_gpu_if_available"] == 1


def test_index_mapping_matches_oracle():
    from bfe_gb300.entry import nds_and_dfs_to_gi
    m = modelgen.coupled_model(W=2e-3, Hw=1e-3, Hs=1e-3, h=0.1e-3, abs_thick=0.3e-3)
    rng = np.random.default_rng(1)
    nds = rng.integers(1, m["gl"].shape[0] + 1, 40)
    dfs = rng.integers(1, m["gl"].shape[1] + 1, 40)
    for a, b in zip(nds_and_dfs_to_gi(nds, dfs, m["gl"]), oentry.nds_and_dfs_to_gi(nds, dfs, m["gl"])):
        assert np.array_equal(a, b)


def test_builder_with_interface_damping_matches_oracle():
    from bfe_gb300.entry import DEFAULT_RUN_OPTIONS, build_matrices
    m = modelgen.coupled_model(W=2e-3, Hw=1e-3, Hs=1e-3, h=0.1e-3, abs_thick=0.3e-3)
    opt = dict(DEFAULT_RUN_OPTIONS, dof_to_use=[1, 2, 4], damping_power_law=2, interface_damping_factor=0.5,
               assemble_on_gpu=False)
    K, C, M, gl = build_matrices(m["mod"], m["matls"], opt)
    Ko, Co, Mo, glo = oassembly.build_global_matrices_v5(m["mod"]["nds"], m["mod"]["els"], m["mod"]["el_mat_i"],
                                                         m["mod"]["el_abs_i"], m["mod"]["el_typ_i"], m["matls"],
                                                         dict(dof_to_use=[1, 2, 4], damping_power_law=2,
                                                              interface_damping_factor=0.5))
    assert np.array_equal(gl, glo)
    for a, b in ((K, Ko), (C, Co), (M, Mo)):
        assert abs(a - b).max() <= 1e-13 * abs(b).max()
    assert abs(C - m["C"]).max() > 0          # the damping was added
