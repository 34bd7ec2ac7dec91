"""Oracle element routines vs golden vectors evaluated from the reference's own
generated element files (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from oracle import elements as E

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "elements_golden.npz"))


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_cpe3_matches_reference_generated_code():
    K, C, M, ln, ld = E.el_CPE3(G["cpe3_nds"], G["cpe3_els"], G["cpe3_D"], float(G["cpe3_rho"]))
    assert _rel(K, G["cpe3_K"]) < 1e-12
    assert _rel(M, G["cpe3_M"]) < 1e-12
    assert np.abs(C).max() == 0 and np.abs(G["cpe3_C"]).max() == 0
    assert ln.tolist() == [1, 1, 1, 2, 2, 2, 3, 3, 3]
    assert ld.tolist() == [1, 2, 3, 1, 2, 3, 1, 2, 3]


def test_cpe3_dof_subset_matches_reference():
    K, C, M, ln, ld = E.el_CPE3(G["cpe3_nds"], G["cpe3_els"], G["cpe3_D"], float(G["cpe3_rho"]), [1, 2])
    keep = [0, 1, 3, 4, 6, 7]
    assert _rel(K, G["cpe3_K"][:, keep][:, :, keep]) < 1e-12
    assert ld.tolist() == [1, 2, 1, 2, 1, 2]


def test_ac2d3_matches_reference_generated_code():
    K, C, M, ln, ld = E.el_AC2D3(G["cpe3_nds"], G["cpe3_els"], G["ac2d3_bulk"], float(G["ac2d3_rho"]))
    assert _rel(K, G["ac2d3_K"]) < 1e-12
    assert _rel(M, G["ac2d3_M"]) < 1e-12
    assert ld.tolist() == [4, 4, 4]


def test_asi2d2_matches_reference_generated_code():
    K, C, M, ln, ld = E.el_ASI2D2(G["asi2d2_nds"], G["asi2d2_els"], np.zeros((6, 6)), 0.0)
    assert _rel(C, G["asi2d2_C"]) < 1e-12
    assert np.abs(K).max() == 0 and np.abs(M).max() == 0
    assert ld.tolist() == [1, 2, 3, 4, 1, 2, 3, 4]


@pytest.mark.parametrize("name", ["CPE3", "AC2D3", "ASI2D2"])
def test_loc_dofs_only_call(name):
    # fn_el_*(...) with empty inputs returns only loc_nd / loc_df (fn_el_CPE3.m:36-44)
    _, _, _, ln, ld = E.ELEMENTS[name](None, None, None, None, [1, 2, 4])
    assert set(ld.tolist()) <= {1, 2, 4}
