"""Synthetic model generation and global assembly (host, vectorised NumPy).

These are the model-preparation utilities a user of the solver runs before
the time march: structured triangle meshes, material regions, fluid-solid
interface elements, absorbing layers, void scatterers, and the v5 global
assembly with the reference's DOF numbering. They follow

    code/fn_rectangular_structured_mesh.m:14-57 (mesh, node/element order)
    code/fn_set_els_inside_bdry_to_mat.m, code/fn_elements_in_region.m
    code/fn_add_fluid_solid_interface_els.m:26-73 (ASI2D2 insertion)
    code/fn_add_absorbing_layer.m:1-17 (absorbing index)
    code/fn_add_scatterer.m:16-20 (void scatterer)
    code/internal/fn_build_global_matrices_v5.m:50-159 (assembly, numbering)
    code/internal/elements/el_builder/el_sym_{CPE3,AC2D3,ASI2D2}.m (elements)

Everything here is vectorised over elements (no per-element Python loops),
so the 1.44M-element benchmark model assembles in seconds. Indices in the
returned model are 1-based like the reference's; gl_lookup holds 1-based
global indices (0 = no DOF).
"""
import numpy as np
import scipy.sparse as sp

TYPE_CODES = {"CPE3": 0, "AC2D3": 1, "ASI2D2": 2}
TYPE_DOFS = {"CPE3": (1, 2, 3), "AC2D3": (4,), "ASI2D2": (1, 2, 3, 4)}


def isotropic_stiffness(E, nu):
    """6x6 isotropic stiffness, engineering shear (fn_isotropic_stiffness_matrix.m:17-23)."""
    lam = E / (1 - 2 * nu) / (1 + nu)
    D = np.zeros((6, 6))
    D[:3, :3] = lam * nu
    D[[0, 1, 2], [0, 1, 2]] = lam * (1 - nu)
    D[[3, 4, 5], [3, 4, 5]] = lam * (1 - 2 * nu) / 2
    return D


def toneburst(t, fc, cycles):
    """-40 dB Gaussian toneburst starting at its 1% envelope point (fn_gaussian_pulse.m:1-15)."""
    t = np.asarray(t, float)
    ct = t.mean()
    T = cycles / (2 * fc * np.sqrt(np.log(100.0)))
    env = np.exp(-((t - ct) / T) ** 2)
    first = int(np.argmax(env > 0.01))
    s = env * np.sin(2 * np.pi * fc * (t - ct))
    return np.concatenate([s[first:], np.zeros(first)])


def rect_mesh(x0, x1, y0, y1, h):
    """Right-isosceles structured mesh with the reference's node and element
    order (column-major node numbering, 'a' triangles then 'b' triangles)."""
    nx = int(np.ceil(abs(x1 - x0) / h)) + 1
    ny = int(np.ceil(abs(y1 - y0) / h)) + 1
    x = np.linspace(x0, x1, nx)
    y = np.linspace(y0, y1, ny)
    nds = np.column_stack([np.repeat(x, ny), np.tile(y, nx)])        # node k = r + c*ny
    r, c = np.meshgrid(np.arange(ny - 1), np.arange(nx - 1), indexing="ij")
    r = r.ravel(order="F")
    c = c.ravel(order="F")
    n00 = r + c * ny + 1
    n10 = (r + 1) + c * ny + 1
    n01 = r + (c + 1) * ny + 1
    n11 = (r + 1) + (c + 1) * ny + 1
    els = np.vstack([np.column_stack([n00, n11, n10]), np.column_stack([n00, n01, n11])])
    return nds, els.astype(np.int64)


def centroids(nds, els):
    """Element centres: mean of each element's node coordinates (zero-padded
    node lists, fn_calc_element_centres.m)."""
    m = (els > 0).sum(1, keepdims=True)
    idx = np.where(els > 0, els, 1) - 1
    return (nds[idx] * (els > 0)[:, :, None]).sum(1) / m


def points_in_polygon(pts, poly):
    """Crossing-number test (boundary points count as inside, like inpolygon)."""
    x, y = pts[:, 0], pts[:, 1]
    inside = np.zeros(x.shape, bool)
    on = np.zeros(x.shape, bool)
    P = np.asarray(poly, float)
    Q = np.roll(P, -1, axis=0)
    scale = max(np.ptp(P[:, 0]), np.ptp(P[:, 1]), 1e-300)
    for (xa, ya), (xb, yb) in zip(P, Q):
        crosses = (ya > y) != (yb > y)
        with np.errstate(divide="ignore", invalid="ignore"):
            xi = xa + (y - ya) * (xb - xa) / (yb - ya)
        inside ^= crosses & (x < xi)
        dx, dy = xb - xa, yb - ya
        L2 = dx * dx + dy * dy
        if L2 > 0:
            t = ((x - xa) * dx + (y - ya) * dy) / L2
            d = np.hypot(x - (xa + t * dx), y - (ya + t * dy))
            on |= (t >= -1e-12) & (t <= 1 + 1e-12) & (d <= 1e-12 * scale)
    return inside | on


def distance_to_polygon(pts, poly):
    """Distance to the nearest polygon vertex or to one of its two adjacent
    edges (fn_dist_point_to_bdry_2D.m:1-69 restricted to that vertex)."""
    P = np.asarray(poly, float)
    nb = P.shape[0]
    d2 = ((pts[:, None, :] - P[None, :, :]) ** 2).sum(-1)
    j = np.argmin(d2, axis=1)
    best = np.sqrt(d2[np.arange(pts.shape[0]), j])
    for step in (1, -1):
        a = P[j]
        b = P[(j + step) % nb]
        ab = b - a
        L = np.sqrt((ab ** 2).sum(1))
        u = ab / L[:, None]
        s = ((pts - a) * u).sum(1)
        perp = np.sqrt((((pts - a) - s[:, None] * u) ** 2).sum(1))
        s = s / L
        best = np.minimum(best, np.where((s < 0) | (s > 1), np.inf, perp))
    return best


def remove_unused_nodes(nds, els):
    """Drop nodes no element uses and renumber the elements' 1-based node
    lists in the original order."""
    used = np.unique(els[els > 0])
    remap = np.zeros(nds.shape[0] + 1, np.int64)
    remap[used] = np.arange(1, used.size + 1)
    return nds[used - 1], remap[els]


def fluid_solid_interfaces(nds, els, typ):
    """ASI2D2 elements on every edge shared by an AC2D3 and a CPE3 element,
    node order chosen so the fluid centroid lies on the side of
    [a_y, -a_x], a = x2 - x1 (fn_add_fluid_solid_interface_els.m:175-195).
    Returns the (n_int, 2) 1-based node pairs in sorted-edge order."""
    tri = np.nonzero(typ != TYPE_CODES["ASI2D2"])[0]
    E = els[tri, :3]
    edges = np.vstack([E[:, [0, 1]], E[:, [1, 2]], E[:, [2, 0]]])
    owner = np.concatenate([tri, tri, tri])
    key_e = np.sort(edges, axis=1)
    key = key_e[:, 0] * (nds.shape[0] + 1) + key_e[:, 1]
    order = np.argsort(key, kind="stable")
    key, owner, key_e = key[order], owner[order], key_e[order]
    same = key[1:] == key[:-1]
    a_el, b_el = owner[:-1][same], owner[1:][same]
    ta, tb = typ[a_el], typ[b_el]
    fl, so = TYPE_CODES["AC2D3"], TYPE_CODES["CPE3"]
    mix = ((ta == fl) & (tb == so)) | ((ta == so) & (tb == fl))
    ed = key_e[:-1][same][mix].copy()
    fluid_el = np.where(ta[mix] == fl, a_el[mix], b_el[mix])
    ctr = centroids(nds, els[fluid_el])
    a = nds[ed[:, 1] - 1] - nds[ed[:, 0] - 1]
    b = np.column_stack([a[:, 1], -a[:, 0]])
    c = ctr - nds[ed[:, 0] - 1]
    flip = (c * b).sum(1) < 0
    ed[flip] = ed[flip][:, ::-1]
    return ed


# ---------------------------------------------------------------------------
# Element matrices (vectorised). Each returns (K, C, M, loc_nd, loc_df) with
# matrices (n_el, ndf, ndf) restricted to the requested DOFs.

def _tri_grads(nds, e):
    x = nds[e[:, :3] - 1, 0]
    y = nds[e[:, :3] - 1, 1]
    J = (x[:, 0] - x[:, 2]) * (y[:, 1] - y[:, 2]) - (x[:, 1] - x[:, 2]) * (y[:, 0] - y[:, 2])
    gx = np.column_stack([y[:, 1] - y[:, 2], y[:, 2] - y[:, 0], y[:, 0] - y[:, 1]]) / J[:, None]
    gy = np.column_stack([x[:, 2] - x[:, 1], x[:, 0] - x[:, 2], x[:, 1] - x[:, 0]]) / J[:, None]
    return J, gx, gy


def _select(dofs_all, nodes_all, keep):
    sel = np.nonzero(np.isin(dofs_all, keep))[0]
    return sel, nodes_all[sel], dofs_all[sel]


def cpe3(nds, e, D, rho, keep):
    """Plane-strain constant-strain triangles (fn_el_CPE3.m:47-155): K = A B'DB
    with the 6 x 6 D and engineering shear, lumped M = rho J / 6 per DOF,
    no C; DOFs of `keep` (1-3) per node, node-major. Returns (K, C, M,
    local node, local DOF) per element."""
    J, gx, gy = _tri_grads(nds, e)
    n = e.shape[0]
    # strain rows [e11, e22, e33, g23, g13, g12]; local dof order (node, dof 1..3)
    B = np.zeros((n, 6, 9))
    for a in range(3):
        B[:, 0, 3 * a] = gx[:, a]
        B[:, 1, 3 * a + 1] = gy[:, a]
        B[:, 3, 3 * a + 2] = gy[:, a]
        B[:, 4, 3 * a + 2] = gx[:, a]
        B[:, 5, 3 * a] = gy[:, a]
        B[:, 5, 3 * a + 1] = gx[:, a]
    sel, ln, ld = _select(np.tile([1, 2, 3], 3), np.repeat([1, 2, 3], 3), keep)
    Bs = B[:, :, sel]
    K = np.matmul(np.matmul(Bs.transpose(0, 2, 1), D), Bs) * (0.5 * J)[:, None, None]
    M = np.zeros_like(K)
    ii = np.arange(sel.size)
    M[:, ii, ii] = (rho * J / 6.0)[:, None]
    return K, np.zeros_like(K), M, ln, ld


def ac2d3(nds, e, bulk, rho, keep):
    """Acoustic pressure triangles (fn_el_AC2D3.m:47-77): K = -(grad N . grad N)
    A / rho, lumped M = -A / (3 bulk), DOF 4 only."""
    J, gx, gy = _tri_grads(nds, e)
    sel, ln, ld = _select(np.array([4, 4, 4]), np.array([1, 2, 3]), keep)
    G = gx[:, :, None] * gx[:, None, :] + gy[:, :, None] * gy[:, None, :]
    K = (-0.5 / rho) * G * J[:, None, None]
    M = np.zeros_like(K)
    ii = np.arange(3)
    M[:, ii, ii] = (-J / (6.0 * bulk))[:, None]
    return K[:, sel][:, :, sel], np.zeros((e.shape[0], sel.size, sel.size)), M[:, sel][:, :, sel], ln, ld


def asi2d2(nds, e, keep):
    """Fluid-solid interface lines (fn_el_ASI2D2.m:49-79): an 8 x 8 C coupling
    the solid DOFs 1-2 of both nodes to the fluid DOF 4 with +-L/4 times the
    unit normal pointing into the fluid; no K or M."""
    p1 = nds[e[:, 0] - 1]
    p2 = nds[e[:, 1] - 1]
    d = p1 - p2
    # -L/4 * unit normal [d_y, -d_x]/L  =  [-d_y, d_x] / 4
    cx = -d[:, 1] / 4.0
    cy = d[:, 0] / 4.0
    n = e.shape[0]
    C = np.zeros((n, 8, 8))
    for s in (0, 4):
        for f in (3, 7):
            C[:, s, f] = C[:, f, s] = cx
            C[:, s + 1, f] = C[:, f, s + 1] = cy
    sel, ln, ld = _select(np.tile([1, 2, 3, 4], 2), np.repeat([1, 2], 4), keep)
    Cs = C[:, sel][:, :, sel]
    return np.zeros_like(Cs), Cs, np.zeros_like(Cs), ln, ld


def assemble(nds, els, el_mat, el_abs, typ, matls, dof_to_use=None, damping_power_law=3,
             max_damping=3.1415e7, max_stiffness_reduction=0.01):
    """Global K, C, M (CSR over the reduced DOFs) and gl_lookup.

    typ holds TYPE_CODES per element; matls is a list of dicts with 'D' (6x6
    or scalar bulk modulus) and 'rho'. Numbering: gi = (node-1)*max_df + dof,
    then DOFs with empty K, M and C columns are removed
    (fn_build_global_matrices_v5.m:127-159, fn_reduce_global_matrices.m:7-22)."""
    names = {v: k for k, v in TYPE_CODES.items()}
    present = sorted({names[c] for c in np.unique(typ)})
    keep = list(dof_to_use) if dof_to_use else None
    dofs_in_use = set()
    for t in present:
        d = np.array(TYPE_DOFS[t])
        dofs_in_use |= set(d[np.isin(d, keep)] if keep else d)
    max_df = max(dofs_in_use)
    n_nodes = nds.shape[0]
    rows, cols, kv, cv, mv = [], [], [], [], []
    for t in present:
        tsel = typ == TYPE_CODES[t]
        for mat in np.unique(el_mat[tsel]):
            es = np.nonzero(tsel & (el_mat == mat))[0]
            e = els[es]
            kd = keep if keep else list(TYPE_DOFS[t])
            if t == "CPE3":
                mt = matls[mat - 1]
                K, C, M, ln, ld = cpe3(nds, e, np.asarray(mt["D"], float), mt["rho"], kd)
            elif t == "AC2D3":
                mt = matls[mat - 1]
                K, C, M, ln, ld = ac2d3(nds, e, float(mt["D"]), mt["rho"], kd)
            else:
                K, C, M, ln, ld = asi2d2(nds, e, kd)
            a = el_abs[es][:, None, None]
            C = C + M * a ** damping_power_law * max_damping
            K = K * np.exp(np.log(max_stiffness_reduction) * a ** (damping_power_law + 1))
            g = (e[:, ln - 1] - 1) * max_df + (ld - 1)                 # (n_el, ndf) 0-based
            ndf = ld.size
            rows.append(np.repeat(g, ndf, axis=1).ravel())             # K(g_c, g_r) += el(r, c)
            cols.append(np.tile(g, (1, ndf)).ravel())
            kv.append(K.transpose(0, 2, 1).ravel())
            cv.append(C.transpose(0, 2, 1).ravel())
            mv.append(M.transpose(0, 2, 1).ravel())
    N = n_nodes * max_df
    r = np.concatenate(rows)
    c = np.concatenate(cols)

    def build(vals):
        # COO triplets summed into CSR (MATLAB sparse), exact zeros dropped
        A = sp.csr_matrix((np.concatenate(vals), (r, c)), shape=(N, N))
        A.sum_duplicates()
        A.eliminate_zeros()
        return A

    K, C, M = build(kv), build(cv), build(mv)
    used = (np.asarray(abs(K).sum(0)).ravel() > 0) | (np.asarray(abs(M).sum(0)).ravel() > 0) | \
        (np.asarray(abs(C).sum(0)).ravel() > 0)
    keep_idx = np.nonzero(used)[0]
    K = K[keep_idx][:, keep_idx].tocsr()
    C = C[keep_idx][:, keep_idx].tocsr()
    M = M[keep_idx][:, keep_idx].tocsr()
    gl = np.zeros((n_nodes, max_df), np.int64)
    gl[keep_idx // max_df, keep_idx % max_df] = np.arange(1, keep_idx.size + 1)
    return K, C, M, gl


def element_stable_dt(nds, els, D, rho, factor=0.9):
    """factor * 2 / sqrt(max eigenvalue of M_e^-1 K_e) over CPE3 elements (in-plane)."""
    K, _, M, _, _ = cpe3(nds, els, D, rho, [1, 2])
    m = np.abs(np.einsum("eii->ei", M))
    s = np.sign(np.einsum("eii->ei", M))
    A = K * s[:, :, None] / np.sqrt(m[:, :, None] * m[:, None, :])
    return factor * 2.0 / np.sqrt(np.linalg.eigvalsh(A).max())


# ---------------------------------------------------------------------------
# Benchmark model families

STEEL = dict(rho=8000.0, E=210e9, nu=0.3)
WATER = dict(rho=1000.0, c=1500.0)


def steel_plate(W=20e-3, H=10e-3, h=0.1e-3, n_mon=16, dof_to_use=(1, 2)):
    """Plain FP64 2D solid workload: rectangular mesh, point force at the
    top-surface centre node (DOF 2), n_mon top-surface monitors."""
    nds, els = rect_mesh(0.0, W, 0.0, H, h)
    D = isotropic_stiffness(STEEL["E"], STEEL["nu"])
    matls = [dict(D=D, rho=STEEL["rho"])]
    ne = els.shape[0]
    typ = np.full(ne, TYPE_CODES["CPE3"])
    K, C, M, gl = assemble(nds, els, np.ones(ne, np.int64), np.zeros(ne), typ, matls, dof_to_use)
    dt = element_stable_dt(nds, els, D, STEEL["rho"])
    top = np.nonzero(np.isclose(nds[:, 1], H))[0]
    src = top[np.argmin(np.abs(nds[top, 0] - W / 2))]
    mon = top[np.linspace(0, top.size - 1, n_mon).astype(int)]
    return dict(nds=nds, els=els, typ=typ, K=K, C=C, M=M, gl=gl, dt=dt,
                src_nodes=[src + 1], src_dof=2, mon_nodes=mon + 1, mon_dof=2)


def smooth_blob(radius, n_harm, amp_max, rng, n_pts=128):
    """Closed curve r(a) = radius * (1 + sum_k A_k sin(k a + phi_k)) / (1 + sum A_k),
    A_k ~ U(0, amp_max), k = 1..n_harm (a seeded smooth random void)."""
    A = rng.uniform(0.0, amp_max, n_harm)
    phi = rng.uniform(0.0, 2 * np.pi, n_harm)
    a = np.linspace(0, 2 * np.pi, n_pts, endpoint=False)
    k = np.arange(1, n_harm + 1)
    r = radius * (1 + (A[None, :] * np.sin(a[:, None] * k[None, :] + phi[None, :])).sum(1)) / (1 + A.sum() / 2)
    return np.column_stack([r * np.cos(a), r * np.sin(a)])


def coupled_water_steel(W=60e-3, H_water=20e-3, H_steel=10e-3, h=0.05e-3, fc=5e6,
                        abs_wavelengths=3.0, blob_radius=1.5e-3, blob_centre=None,
                        seed=0, dof_to_use=(1, 2, 4), damping_power_law=2,
                        array_elements=64, array_pitch=0.6e-3, element_width=None,
                        blob_polygon_pts=None):
    """Coupled water-over-steel workload: ASI2D2 interface, absorbing layers
    (left, right, bottom; thickness in steel longitudinal wavelengths,
    quadratic grading), a void in the steel (the given polygon, or a seeded
    smooth blob), and a linear array on the top (water) surface whose
    elements are the sources/receivers."""
    nds, els = rect_mesh(0.0, W, 0.0, H_water + H_steel, h)
    D = isotropic_stiffness(STEEL["E"], STEEL["nu"])
    bulk = WATER["c"] ** 2 * WATER["rho"]
    matls = [dict(D=D, rho=STEEL["rho"]), dict(D=bulk, rho=WATER["rho"])]
    ctr = centroids(nds, els)
    el_mat = np.where(ctr[:, 1] > H_steel, 2, 1).astype(np.int64)
    rng = np.random.default_rng(seed)
    blob = None
    if blob_polygon_pts is not None:
        blob = np.asarray(blob_polygon_pts, float)
    elif blob_radius > 0:
        bc = np.array(blob_centre if blob_centre is not None else (W / 2, H_steel / 2))
        blob = smooth_blob(blob_radius, 8, 0.2, rng) + bc
    if blob is not None:
        keep = ~points_in_polygon(ctr, blob)
        els, el_mat = els[keep], el_mat[keep]
        nds, els = remove_unused_nodes(nds, els)
        ctr = centroids(nds, els)
    cL = np.sqrt(D[0, 0] / STEEL["rho"])
    thick = abs_wavelengths * cL / fc
    Htot = H_water + H_steel
    inner = np.array([[thick, thick], [W - thick, thick], [W - thick, Htot + 1.0], [thick, Htot + 1.0]])
    el_abs = np.clip(distance_to_polygon(ctr, inner) / thick, 0.0, 1.0)
    el_abs[points_in_polygon(ctr, inner)] = 0.0
    typ = np.where(el_mat == 2, TYPE_CODES["AC2D3"], TYPE_CODES["CPE3"])
    ed = fluid_solid_interfaces(nds, els, typ)
    els_all = np.vstack([els, np.column_stack([ed, np.zeros(ed.shape[0], np.int64)])])
    typ = np.concatenate([typ, np.full(ed.shape[0], TYPE_CODES["ASI2D2"])])
    el_mat = np.concatenate([el_mat, np.zeros(ed.shape[0], np.int64)])
    el_abs = np.concatenate([el_abs, np.zeros(ed.shape[0])])
    K, C, M, gl = assemble(nds, els_all, el_mat, el_abs, typ, matls, dof_to_use,
                           damping_power_law=damping_power_law)
    solid = typ == TYPE_CODES["CPE3"]
    dt = element_stable_dt(nds, els_all[solid, :3], D, STEEL["rho"])
    # linear array on the top surface (water): element e covers
    # [x_e - w/2, x_e + w/2] around x_e = W/2 + (e - (n-1)/2) * pitch
    top = np.nonzero(np.isclose(nds[:, 1], Htot))[0]
    width = element_width if element_width is not None else 0.8 * array_pitch
    xc = W / 2 + (np.arange(array_elements) - (array_elements - 1) / 2) * array_pitch
    src_nodes = [top[np.abs(nds[top, 0] - x) <= width / 2 + 1e-12] + 1 for x in xc]
    centre_nodes = np.array([top[np.argmin(np.abs(nds[top, 0] - x))] + 1 for x in xc])
    return dict(nds=nds, els=els_all, typ=typ, el_mat=el_mat, el_abs=el_abs, K=K, C=C, M=M,
                gl=gl, dt=dt, src_nodes=src_nodes, src_dof=4, mon_nodes=centre_nodes,
                mon_dof=4, matls=matls, n_interface=ed.shape[0])


def steel_subdomain(side, h=0.05e-3, fc=5e6, seed=0, n_src=64, n_mon=64, abs_wavelengths=3.0,
                    blob_radius=1.5e-3, dof_to_use=(1, 2), damping_power_law=2):
    """Square steel scatterer sub-domain model: absorbing layers on all four
    sides (thickness min(3 wavelengths, side / 4), quadratic grading), a seeded
    smooth void at the centre, n_src point sources (DOF 2) and n_mon monitors
    (DOF 2) spread along a line just inside the absorbing frame, near its top."""
    rng = np.random.default_rng(seed)
    nds, els = rect_mesh(0.0, side, 0.0, side, h)
    D = isotropic_stiffness(STEEL["E"], STEEL["nu"])
    matls = [dict(D=D, rho=STEEL["rho"])]
    ctr = centroids(nds, els)
    r = min(blob_radius, side / 8)
    blob = smooth_blob(r, 8, 0.2, rng) + np.array([side / 2, side / 2])
    keep = ~points_in_polygon(ctr, blob)
    els = els[keep]
    nds, els = remove_unused_nodes(nds, els)
    ctr = centroids(nds, els)
    cL = np.sqrt(D[0, 0] / STEEL["rho"])
    thick = min(abs_wavelengths * cL / fc, side / 4)
    inner = np.array([[thick, thick], [side - thick, thick], [side - thick, side - thick],
                      [thick, side - thick]])
    el_abs = np.clip(distance_to_polygon(ctr, inner) / thick, 0.0, 1.0)
    el_abs[points_in_polygon(ctr, inner)] = 0.0
    ne = els.shape[0]
    typ = np.full(ne, TYPE_CODES["CPE3"])
    K, C, M, gl = assemble(nds, els, np.ones(ne, np.int64), el_abs, typ, matls, dof_to_use,
                           damping_power_law=damping_power_law)
    dt = element_stable_dt(nds, els, D, STEEL["rho"])
    # transducer line just inside the absorbing frame (the driven boundary of
    # a sub-domain lies inside its absorbers, subdoms/fn_create_subdomain.m)
    y_line = side - thick - 2 * h
    row = np.abs(nds[:, 1] - y_line)
    line = np.nonzero(row <= row.min() + 1e-12)[0]
    line = line[(nds[line, 0] >= thick + 2 * h) & (nds[line, 0] <= side - thick - 2 * h)]
    line = line[np.argsort(nds[line, 0])]
    src = line[np.linspace(0, line.size - 1, n_src).astype(int)] + 1
    mon = line[np.linspace(0, line.size - 1, n_mon).astype(int)] + 1
    return dict(nds=nds, els=els, K=K, C=C, M=M, gl=gl, dt=dt, src_nodes=[[s] for s in src],
                src_dof=2, mon_nodes=mon, mon_dof=2)


def subdomain_sides(n_models, dof_min=50e3, dof_max=400e3, h=0.05e-3, seed=1, dofs_per_node=2):
    """Side lengths of square models whose DOF counts are log-uniform in
    [dof_min, dof_max] (seeded)."""
    rng = np.random.default_rng(seed)
    dof = np.exp(rng.uniform(np.log(dof_min), np.log(dof_max), n_models))
    nodes_per_side = np.sqrt(dof / dofs_per_node)
    return (nodes_per_side - 1) * h


def global_indices(gl, nodes, dof):
    """1-based global indices of (node, dof) pairs that exist (fn_BristolFE_v2.m:159-168)."""
    g = gl[np.asarray(nodes, np.int64) - 1, dof - 1]
    return g[g > 0]


# ---------------------------------------------------------------------------
# 3D structured solid (8-node bricks)

_BRICK = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                   [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], np.int64)


def brick_matrices(dx, dy, dz, D, rho):
    """Stiffness (24 x 24, node-major, DOF-minor) and lumped nodal mass of one
    trilinear brick of sides dx, dy, dz: 2 x 2 x 2 Gauss integration of
    B' D B with the Voigt order [11, 22, 33, 23, 13, 12] (engineering shear);
    lumped mass = rho * V / 8 per node."""
    g = 1.0 / np.sqrt(3.0)
    sgn = 2 * _BRICK - 1                           # natural coordinates of the nodes
    h = np.array([dx, dy, dz], float)
    K = np.zeros((24, 24))
    detJ = dx * dy * dz / 8.0
    for q in np.array(np.meshgrid([-g, g], [-g, g], [-g, g], indexing="ij")).reshape(3, -1).T:
        # dN/dx_d = sgn_d * prod_{e != d}(1 + sgn_e q_e) / 8 * (2 / h_d)
        f = 1 + sgn * q
        dN = np.stack([sgn[:, d] * np.prod(np.delete(f, d, axis=1), axis=1) / 8 * (2 / h[d])
                       for d in range(3)], axis=1)                    # (8, 3)
        B = np.zeros((6, 24))
        for a in range(8):
            c = 3 * a
            B[0, c], B[1, c + 1], B[2, c + 2] = dN[a]
            B[3, c + 1], B[3, c + 2] = dN[a, 2], dN[a, 1]
            B[4, c], B[4, c + 2] = dN[a, 2], dN[a, 0]
            B[5, c], B[5, c + 1] = dN[a, 1], dN[a, 0]
        K += B.T @ D @ B * detJ
    return K, rho * dx * dy * dz / 8.0


def cubic_mesh(x1, y1, z1, h):
    """Node and brick layout of a structured box [0, x1] x [0, y1] x [0, z1]
    with the reference's ordering (fn_3d_cubic_structured_mesh.m: node
    index i + nx (j + ny k), 1-based, bricks i fastest)."""
    sz = np.array([x1, y1, z1], float)
    n = (np.ceil(sz / h) + 1).astype(np.int64)
    d = sz / (n - 1)
    i, j, k = np.meshgrid(np.arange(n[0]), np.arange(n[1]), np.arange(n[2]), indexing="ij")
    nds = np.column_stack([i.ravel(order="F") * d[0], j.ravel(order="F") * d[1], k.ravel(order="F") * d[2]])
    ei, ej, ek = np.meshgrid(np.arange(n[0] - 1), np.arange(n[1] - 1), np.arange(n[2] - 1), indexing="ij")
    ei, ej, ek = (x.ravel(order="F") for x in (ei, ej, ek))
    els = np.column_stack([(ei + o[0]) + n[0] * ((ej + o[1]) + n[1] * (ek + o[2])) + 1 for o in _BRICK])
    return nds, els, n, d


def assemble_brick_grid(n, d, D, rho, el_abs, damping_power_law=3, max_damping=3.1415e7,
                        max_stiffness_reduction=0.01):
    """Global K, C, M (CSR, DOF = 3 node + dof) of a structured brick grid with
    per-element absorbing index el_abs (grid order). Every brick shares one
    element matrix; the absorbing grading scales it per element
    (fn_build_global_matrices_v5.m:115-116), so K is accumulated as 27-point
    node-block stencils with array slices instead of a COO sort."""
    nx, ny, nz = (int(v) for v in n)
    ke, me = brick_matrices(d[0], d[1], d[2], D, rho)
    a = np.asarray(el_abs, float).reshape(nx - 1, ny - 1, nz - 1, order="F")
    s = np.exp(np.log(max_stiffness_reduction) * a ** (damping_power_law + 1))
    cfac = a ** damping_power_law * max_damping
    Kb = np.zeros((nx, ny, nz, 27, 3, 3))
    mn = np.zeros((nx, ny, nz))
    cn = np.zeros((nx, ny, nz))
    for ia, oa in enumerate(_BRICK):
        sa = (slice(oa[0], oa[0] + nx - 1), slice(oa[1], oa[1] + ny - 1), slice(oa[2], oa[2] + nz - 1))
        mn[sa] += me
        cn[sa] += me * cfac
        for ib, ob in enumerate(_BRICK):
            off = ob - oa
            slot = (off[0] + 1) + 3 * (off[1] + 1) + 9 * (off[2] + 1)
            Kb[sa + (slot,)] += s[..., None, None] * ke[3 * ia:3 * ia + 3, 3 * ib:3 * ib + 3]
    # CSR rows: node-major, dof-minor; columns sorted (neighbour node index, dof)
    nn = nx * ny * nz
    node = np.arange(nn)
    ci, cj, ck = node % nx, (node // nx) % ny, node // (nx * ny)
    Kf = Kb.reshape(nx * ny * nz, 27, 3, 3, order="F")
    rows, cols, vals = [], [], []
    for slot in range(27):
        o = np.array([slot % 3 - 1, (slot // 3) % 3 - 1, slot // 9 - 1])
        ok = (ci + o[0] >= 0) & (ci + o[0] < nx) & (cj + o[1] >= 0) & (cj + o[1] < ny) & \
             (ck + o[2] >= 0) & (ck + o[2] < nz)
        src = node[ok]
        nb = src + o[0] + nx * (o[1] + ny * o[2])
        blk = Kf[src, slot]                                       # (m, 3, 3)
        for r in range(3):
            for c in range(3):
                rows.append(3 * src + r)
                cols.append(3 * nb + c)
                vals.append(blk[:, r, c])
    N = 3 * nn
    K = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(N, N))
    K.sum_duplicates()
    K.eliminate_zeros()
    mvec = np.repeat(mn.ravel(order="F"), 3)
    cvec = np.repeat(cn.ravel(order="F"), 3)
    M = sp.diags(mvec).tocsr()
    C = sp.diags(cvec).tocsr()
    C.eliminate_zeros()
    gl = (3 * node[:, None] + np.arange(3)[None, :] + 1).astype(np.int64)
    return K, C, M, gl


def box_distance(pts, lo, hi):
    """Euclidean distance from points to an axis-aligned box (0 inside)."""
    dlo = np.maximum(lo - pts, 0.0)
    dhi = np.maximum(pts - hi, 0.0)
    return np.sqrt(((dlo + dhi) ** 2).sum(1))


def steel_block_3d(Lx=10e-3, Ly=10e-3, Lz=5e-3, h=0.1e-3, fc=5e6, abs_wavelengths=3.0,
                   n_mon=64, damping_power_law=3):
    """3D steel block of 8-node bricks: absorbing layers on the four sides and
    the bottom (thickness in longitudinal wavelengths, capped at a quarter of
    the smaller side), a point force normal to the top face (DOF 3) at its
    centre, n_mon monitors on a square grid of top-face nodes."""
    nds, els, n, d = cubic_mesh(Lx, Ly, Lz, h)
    D = isotropic_stiffness(STEEL["E"], STEEL["nu"])
    cL = np.sqrt(D[0, 0] / STEEL["rho"])
    thick = min(abs_wavelengths * cL / fc, min(Lx, Ly) / 4, Lz / 2)
    ctr = centroids(nds, els)
    lo = np.array([thick, thick, thick])
    hi = np.array([Lx - thick, Ly - thick, np.inf])
    el_abs = np.clip(box_distance(ctr, lo, hi) / thick, 0.0, 1.0)
    K, C, M, gl = assemble_brick_grid(n, d, D, STEEL["rho"], el_abs, damping_power_law)
    ke, me = brick_matrices(d[0], d[1], d[2], D, STEEL["rho"])
    lam = np.linalg.eigvalsh(ke / me).max()
    dt = 0.9 * 2.0 / np.sqrt(lam)
    top = np.nonzero(np.isclose(nds[:, 2], Lz))[0]
    src = top[np.argmin((nds[top, 0] - Lx / 2) ** 2 + (nds[top, 1] - Ly / 2) ** 2)]
    side = int(round(np.sqrt(n_mon)))
    gx = np.linspace(thick, Lx - thick, side)
    gy = np.linspace(thick, Ly - thick, side)
    mon = np.array([top[np.argmin((nds[top, 0] - x) ** 2 + (nds[top, 1] - y) ** 2)]
                    for y in gy for x in gx]) + 1
    return dict(nds=nds, els=els, el_abs=el_abs, K=K, C=C, M=M, gl=gl, dt=dt,
                src_nodes=[src + 1], src_dof=3, mon_nodes=mon, mon_dof=3)


# ---------------------------------------------------------------------------
# Element data for adjoint gradients

def cpe3_element_data(nds, els, el_abs, D, rho, gl, dof_to_use=(1, 2), damping_power_law=3,
                      max_damping=3.1415e7, max_stiffness_reduction=0.01):
    """Per-element data of a CPE3 model for bfe_adjoint_gradient: stiffness at
    unit scale with the absorbing grading, lumped mass and damping per unit
    density (fn_build_global_matrices_v5.m:115-116), 0-based global rows."""
    K, _, M, ln, ld = cpe3(nds, els, D, rho, list(dof_to_use))
    a = np.asarray(el_abs, float)
    K = K * np.exp(np.log(max_stiffness_reduction) * a ** (damping_power_law + 1))[:, None, None]
    mh = np.einsum("eii->ei", M) / rho
    ch = mh * (a ** damping_power_law * max_damping)[:, None]
    dof = gl[els[:, ln - 1] - 1, ld - 1] - 1
    return K, mh, ch, dof


def assemble_from_elements(ke, mh, ch, dof, n, s=None, rho=None):
    """K = sum s_e K_e, M = diag(sum rho_e Mh_e), C = diag(sum rho_e Ch_e)."""
    n_el, ndf = dof.shape
    s = np.ones(n_el) if s is None else np.asarray(s, float)
    rho = np.ones(n_el) if rho is None else np.asarray(rho, float)
    r = np.repeat(dof, ndf, axis=1).ravel()
    c = np.tile(dof, (1, ndf)).ravel()
    K = sp.csr_matrix(((ke * s[:, None, None]).transpose(0, 2, 1).ravel(), (r, c)), shape=(n, n))
    K.sum_duplicates()
    m = np.bincount(dof.ravel(), (mh * rho[:, None]).ravel(), minlength=n)
    cc = np.bincount(dof.ravel(), (ch * rho[:, None]).ravel(), minlength=n)
    return K, sp.diags(cc).tocsr(), sp.diags(m).tocsr()


def steel_plate_adjoint(W=30e-3, H=15e-3, h=0.05e-3, fc=5e6, n_src=16, n_rec=16, abs_wavelengths=3.0,
                        damping_power_law=3, seed=2, bump_width=1e-3, n_bumps=12, amplitude=0.05):
    """Adjoint benchmark model: steel plate with absorbing layers on the
    sides and bottom, n_src point sources and n_rec receivers (DOF 2) spread
    along the top surface inside the absorbers, and a seeded target stiffness
    field 1 + sum of Gaussian bumps (width bump_width, clipped to
    +-amplitude) for generating observed A-scans."""
    nds, els = rect_mesh(0.0, W, 0.0, H, h)
    D = isotropic_stiffness(STEEL["E"], STEEL["nu"])
    rho = STEEL["rho"]
    ctr = centroids(nds, els)
    cL = np.sqrt(D[0, 0] / rho)
    thick = min(abs_wavelengths * cL / fc, W / 4, H / 2)
    inner = np.array([[thick, thick], [W - thick, thick], [W - thick, H + 1.0], [thick, H + 1.0]])
    el_abs = np.clip(distance_to_polygon(ctr, inner) / thick, 0.0, 1.0)
    el_abs[points_in_polygon(ctr, inner)] = 0.0
    ne = els.shape[0]
    typ = np.full(ne, TYPE_CODES["CPE3"])
    K, C, M, gl = assemble(nds, els, np.ones(ne, np.int64), el_abs, typ, [dict(D=D, rho=rho)], (1, 2),
                           damping_power_law=damping_power_law)
    dt = element_stable_dt(nds, els, D, rho)
    ed = cpe3_element_data(nds, els, el_abs, D, rho, gl, (1, 2), damping_power_law)
    rng = np.random.default_rng(seed)
    cx = rng.uniform(thick, W - thick, n_bumps)
    cy = rng.uniform(thick, H - 2 * h, n_bumps)
    amp = rng.uniform(-1.0, 1.0, n_bumps)
    field = np.zeros(ne)
    for x0, y0, a0 in zip(cx, cy, amp):
        field += a0 * np.exp(-((ctr[:, 0] - x0) ** 2 + (ctr[:, 1] - y0) ** 2) / (2 * bump_width ** 2))
    s_true = 1 + np.clip(amplitude * field, -amplitude, amplitude)
    top = np.nonzero(np.isclose(nds[:, 1], H))[0]
    top = top[(nds[top, 0] >= thick) & (nds[top, 0] <= W - thick)]
    top = top[np.argsort(nds[top, 0])]
    src = top[np.linspace(0, top.size - 1, n_src).astype(int)] + 1
    rec = top[np.linspace(0, top.size - 1, n_rec).astype(int)] + 1
    return dict(nds=nds, els=els, el_abs=el_abs, K=K, C=C, M=M, gl=gl, dt=dt, element_data=ed,
                s_true=s_true, rho=rho, src_nodes=[[x] for x in src], rec_nodes=rec)
