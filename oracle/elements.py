"""Element matrix restatements (FP64, NumPy) - oracle only.

Each routine returns (el_K, el_C, el_M, loc_nd, loc_df) with element matrices
shaped (n_els, ndf, ndf), like the reference's generated ``fn_el_*.m`` files.
They are derived here from the element definitions in the reference's
symbolic builder (``code/internal/elements/el_builder/el_sym_*.m``), not
transcribed from the generated expressions; the golden vectors in
``tests/golden`` check them against the generated files' own values.
"""
import numpy as np

# loc_nd / loc_df orders of the reference element files
_CPE3_LOC_ND = np.array([1, 1, 1, 2, 2, 2, 3, 3, 3])
_CPE3_LOC_DF = np.array([1, 2, 3, 1, 2, 3, 1, 2, 3])   # fn_el_CPE3.m:26-29
_AC2D3_LOC_ND = np.array([1, 2, 3])
_AC2D3_LOC_DF = np.array([4, 4, 4])                    # fn_el_AC2D3.m:26-29
_ASI2D2_LOC_ND = np.array([1, 1, 1, 1, 2, 2, 2, 2])
_ASI2D2_LOC_DF = np.array([1, 2, 3, 4, 1, 2, 3, 4])    # fn_el_ASI2D2.m:26-29
_HEX8_LOC_ND = np.repeat(np.arange(1, 9), 3)
_HEX8_LOC_DF = np.tile(np.array([1, 2, 3]), 8)


def _remove_dofs(loc_nd, loc_df, dofs_to_use, *mats):
    """fn_remove_dofs_from_el_matrices.m:1-19."""
    if dofs_to_use is None or len(dofs_to_use) == 0:
        dofs_to_use = np.unique(loc_df)
    j = np.isin(loc_df, dofs_to_use)
    out = [m[:, j][:, :, j] for m in mats]
    return (loc_nd[j], loc_df[j], *out)


def _tri_geometry(nds, els):
    """Signed detJ and shape-function gradients of a linear triangle.

    Shape functions n1 = q1, n2 = q2, n3 = 1 - q1 - q2 (el_sym_CPE3.m:50-53);
    detJ is the determinant of d(x, y)/d(q1, q2) and is NOT made positive,
    as in the reference (fn_el_CPE3.m:56).
    """
    x1, y1 = nds[els[:, 0] - 1, 0], nds[els[:, 0] - 1, 1]
    x2, y2 = nds[els[:, 1] - 1, 0], nds[els[:, 1] - 1, 1]
    x3, y3 = nds[els[:, 2] - 1, 0], nds[els[:, 2] - 1, 1]
    J = (x1 - x3) * (y2 - y3) - (x2 - x3) * (y1 - y3)
    dndx = np.stack([y2 - y3, y3 - y1, y1 - y2], axis=1) / J[:, None]
    dndy = np.stack([x3 - x2, x1 - x3, x2 - x1], axis=1) / J[:, None]
    return J, dndx, dndy


def el_CPE3(nds, els, D, rho, dofs_to_use=None):
    """Plane-strain constant-strain triangle (el_sym_CPE3.m:28-85).

    Strain vector (engineering shear), per the reference's diff_matrix
    (el_sym_CPE3.m:58-64) with no z-derivatives in 2D:
    [du1/dx, du2/dy, 0, du3/dy, du3/dx, du1/dy + du2/dx].
    K = B' D B * detJ / 2 (integral over the unit triangle), lumped
    M = diag(rho * detJ / 6) (el_sym_CPE3.m:75-76).
    """
    loc_nd, loc_df = _CPE3_LOC_ND.copy(), _CPE3_LOC_DF.copy()
    if nds is None or els is None or D is None or rho is None:
        ln, ld = _remove_dofs(loc_nd, loc_df, dofs_to_use)
        return None, None, None, ln, ld
    els = np.asarray(els)
    n = els.shape[0]
    J, bx, by = _tri_geometry(nds, els)
    B = np.zeros((n, 6, 9))
    for a in range(3):
        c = 3 * a
        B[:, 0, c + 0] = bx[:, a]
        B[:, 1, c + 1] = by[:, a]
        B[:, 3, c + 2] = by[:, a]
        B[:, 4, c + 2] = bx[:, a]
        B[:, 5, c + 0] = by[:, a]
        B[:, 5, c + 1] = bx[:, a]
    D = np.asarray(D, float)
    K = np.einsum("eki,kl,elj->eij", B, D, B) * (J / 2)[:, None, None]
    M = np.zeros((n, 9, 9))
    idx = np.arange(9)
    M[:, idx, idx] = (J * rho / 6)[:, None]
    C = np.zeros((n, 9, 9))
    Kr, Cr, Mr = _remove_dofs(loc_nd, loc_df, dofs_to_use, K, C, M)[2:]
    ln, ld = _remove_dofs(loc_nd, loc_df, dofs_to_use)
    return Kr, Cr, Mr, ln, ld


def el_AC2D3(nds, els, D, rho, dofs_to_use=None):
    """Acoustic pressure triangle (el_sym_AC2D3.m:175-239).

    K = -(grad N' grad N) * detJ / 2 / rho and lumped M = -detJ / 6 / bulk,
    with D the scalar bulk modulus (el_sym_AC2D3.m:214-231); DOF index 4.
    """
    loc_nd, loc_df = _AC2D3_LOC_ND.copy(), _AC2D3_LOC_DF.copy()
    if nds is None or els is None or D is None or rho is None:
        ln, ld = _remove_dofs(loc_nd, loc_df, dofs_to_use)
        return None, None, None, ln, ld
    els = np.asarray(els)
    n = els.shape[0]
    J, bx, by = _tri_geometry(nds, els)
    G = bx[:, :, None] * bx[:, None, :] + by[:, :, None] * by[:, None, :]
    D = float(np.asarray(D).ravel()[0])
    K = -G * (J / 2)[:, None, None] / rho
    M = np.zeros((n, 3, 3))
    idx = np.arange(3)
    M[:, idx, idx] = (-J / (6 * D))[:, None]
    C = np.zeros((n, 3, 3))
    Kr, Cr, Mr = _remove_dofs(loc_nd, loc_df, dofs_to_use, K, C, M)[2:]
    ln, ld = _remove_dofs(loc_nd, loc_df, dofs_to_use)
    return Kr, Cr, Mr, ln, ld


def el_ASI2D2(nds, els, D, rho, dofs_to_use=None):
    """Fluid-solid interface line element (el_sym_ASI2D2.m:269-311).

    tmp = x1 - x2, L = |tmp|, unit normal nrm = [tmp_y, -tmp_x] / L.
    The coupling sits in C only: C(solid dof k of node a, fluid dof of
    node b) = -L / 4 * nrm_k for k in {1, 2}, a, b in {1, 2}, and the
    transposed block (chosen variant, el_sym_ASI2D2.m:308-310).
    """
    loc_nd, loc_df = _ASI2D2_LOC_ND.copy(), _ASI2D2_LOC_DF.copy()
    if nds is None or els is None or D is None or rho is None:
        ln, ld = _remove_dofs(loc_nd, loc_df, dofs_to_use)
        return None, None, None, ln, ld
    els = np.asarray(els)
    n = els.shape[0]
    p1 = nds[els[:, 0] - 1]
    p2 = nds[els[:, 1] - 1]
    tmp = p1 - p2
    L = np.sqrt((tmp ** 2).sum(1))
    nrm = np.stack([tmp[:, 1], -tmp[:, 0]], 1) / L[:, None]
    C = np.zeros((n, 8, 8))
    for a in (0, 4):           # node-a solid dofs 1, 2 at local rows a, a+1
        for b in (3, 7):       # fluid dof of node b at local col b
            C[:, a + 0, b] = -L / 4 * nrm[:, 0]
            C[:, a + 1, b] = -L / 4 * nrm[:, 1]
            C[:, b, a + 0] = -L / 4 * nrm[:, 0]
            C[:, b, a + 1] = -L / 4 * nrm[:, 1]
    K = np.zeros((n, 8, 8))
    M = np.zeros((n, 8, 8))
    Kr, Cr, Mr = _remove_dofs(loc_nd, loc_df, dofs_to_use, K, C, M)[2:]
    ln, ld = _remove_dofs(loc_nd, loc_df, dofs_to_use)
    return Kr, Cr, Mr, ln, ld


_HEX_NAT = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                     [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], float)


def el_HEX8(nds, els, D, rho, dofs_to_use=None):
    """8-node trilinear brick (no reference counterpart; the reference names
    C3D8R only for external solvers, examples/solid_example_3d.m:18).

    Full 2x2x2 Gauss integration of K = int B' D B dV with the same Voigt
    order as the reference's solid elements ([11, 22, 33, 23, 13, 12],
    engineering shear, el_sym_CPE3.m:58-64), and a lumped mass equal to the
    row sums of the consistent mass (rho * V / 8 per node for a
    parallelepiped).
    """
    loc_nd, loc_df = _HEX8_LOC_ND.copy(), _HEX8_LOC_DF.copy()
    if nds is None or els is None or D is None or rho is None:
        ln, ld = _remove_dofs(loc_nd, loc_df, dofs_to_use)
        return None, None, None, ln, ld
    els = np.asarray(els)
    n = els.shape[0]
    X = nds[els - 1]                        # (n, 8, 3)
    g = 1.0 / np.sqrt(3.0)
    K = np.zeros((n, 24, 24))
    Mc = np.zeros((n, 8))
    D = np.asarray(D, float)
    for xi in (-g, g):
        for eta in (-g, g):
            for zeta in (-g, g):
                q = np.array([xi, eta, zeta])
                Nn = np.prod(1 + _HEX_NAT * q, axis=1) / 8          # (8,)
                dN = np.zeros((8, 3))
                for d in range(3):
                    o = [k for k in range(3) if k != d]
                    dN[:, d] = _HEX_NAT[:, d] * (1 + _HEX_NAT[:, o[0]] * q[o[0]]) * \
                        (1 + _HEX_NAT[:, o[1]] * q[o[1]]) / 8
                Jm = np.einsum("ad,eak->ekd", dN, X)                 # dx_k/dq_d
                detJ = np.linalg.det(Jm)
                dNx = np.einsum("ad,edk->eak", dN, np.linalg.inv(Jm))  # dN/dx_k
                B = np.zeros((n, 6, 24))
                for a in range(8):
                    c = 3 * a
                    B[:, 0, c + 0] = dNx[:, a, 0]
                    B[:, 1, c + 1] = dNx[:, a, 1]
                    B[:, 2, c + 2] = dNx[:, a, 2]
                    B[:, 3, c + 1] = dNx[:, a, 2]
                    B[:, 3, c + 2] = dNx[:, a, 1]
                    B[:, 4, c + 0] = dNx[:, a, 2]
                    B[:, 4, c + 2] = dNx[:, a, 0]
                    B[:, 5, c + 0] = dNx[:, a, 1]
                    B[:, 5, c + 1] = dNx[:, a, 0]
                K += np.einsum("eki,kl,elj->eij", B, D, B) * detJ[:, None, None]
                Mc += rho * Nn[None, :] * detJ[:, None]   # row sums of N'N
    M = np.zeros((n, 24, 24))
    idx = np.arange(24)
    M[:, idx, idx] = np.repeat(Mc, 3, axis=1)
    C = np.zeros((n, 24, 24))
    Kr, Cr, Mr = _remove_dofs(loc_nd, loc_df, dofs_to_use, K, C, M)[2:]
    ln, ld = _remove_dofs(loc_nd, loc_df, dofs_to_use)
    return Kr, Cr, Mr, ln, ld


ELEMENTS = {"CPE3": el_CPE3, "AC2D3": el_AC2D3, "ASI2D2": el_ASI2D2, "HEX8": el_HEX8}
