"""Mesh and model-setup restatements (FP64, NumPy) - oracle only.

Conventions follow the reference: node coordinates are an (n_nds, dims)
array, element connectivity ``els`` is 1-based with 0 padding, materials are
1-based (0 = no material, used by interface elements), element types are
strings ('CPE3', 'AC2D3', 'ASI2D2', and the added 'HEX8').
"""
import numpy as np


def _mgrid_numbers(ny, nx):
    """node_numbers = reshape(1:N, ny, nx) of the reference (column-major)."""
    return np.arange(1, ny * nx + 1, dtype=np.int64).reshape(nx, ny).T


def _colvec(a):
    """MATLAB a(:) (column-major flatten)."""
    return np.asarray(a).flatten(order="F")


def inpolygon(px, py, poly):
    """Points inside or on the boundary of a closed polygon (MATLAB inpolygon).

    Even-odd crossing rule plus an on-edge test, as MATLAB's inpolygon
    reports edge points as inside.
    """
    px = np.asarray(px, float)
    py = np.asarray(py, float)
    poly = np.asarray(poly, float)
    x0, y0 = poly[:, 0], poly[:, 1]
    x1, y1 = np.roll(x0, -1), np.roll(y0, -1)
    inside = np.zeros(px.shape, bool)
    on = np.zeros(px.shape, bool)
    scale = max(np.ptp(x0), np.ptp(y0), 1e-300)
    tol = 1e-12 * scale
    for k in range(len(x0)):
        xa, ya, xb, yb = x0[k], y0[k], x1[k], y1[k]
        cond = (ya > py) != (yb > py)
        with np.errstate(divide="ignore", invalid="ignore"):
            xint = xa + (py - ya) * (xb - xa) / (yb - ya)
        inside ^= cond & (px < xint)
        # on-edge test
        dx, dy = xb - xa, yb - ya
        L2 = dx * dx + dy * dy
        if L2 > 0:
            t = ((px - xa) * dx + (py - ya) * dy) / L2
            cx, cy = xa + t * dx, ya + t * dy
            d = np.hypot(px - cx, py - cy)
            on |= (t >= -1e-12) & (t <= 1 + 1e-12) & (d <= tol)
    return inside | on


def calc_element_centres(nds, els):
    """fn_calc_element_centres.m:1-18 (mean of the non-zero element nodes)."""
    els = np.asarray(els)
    ctr = np.zeros((els.shape[0], nds.shape[1]))
    n = np.zeros((els.shape[0], 1))
    for i in range(els.shape[1]):
        j = els[:, i]
        v = (j > 0)[:, None]
        n = n + v
        jj = np.where(j > 0, j, 1) - 1
        ctr = ctr + nds[jj, :] * v
    return ctr / n


def elements_in_region(nds, els, region):
    """fn_elements_in_region.m:1-8 - element centroids inside polygon."""
    c = calc_element_centres(nds, els)
    inn = inpolygon(c[:, 0], c[:, 1], region)
    return inn, ~inn


def remove_unused_nodes(nds, els):
    """fn_remove_unused_nodes.m:1-19; returns (nds2, els2, old_nds 1-based)."""
    els = np.asarray(els, dtype=np.int64)
    used = np.unique(els[els > 0])
    new_of_old = np.zeros(nds.shape[0] + 1, dtype=np.int64)
    new_of_old[used] = np.arange(1, used.size + 1)
    els2 = new_of_old[els]            # 0 padding maps to 0
    return nds[used - 1, :], els2, used


def rectangular_structured_mesh(bdry_pts, el_size):
    """fn_rectangular_structured_mesh.m:14-57 (right-isosceles triangles)."""
    bdry_pts = np.asarray(bdry_pts, float)
    lo, hi = bdry_pts.min(0), bdry_pts.max(0)
    bx, by = abs(hi[0] - lo[0]), abs(hi[1] - lo[1])
    nx = int(np.ceil(bx / el_size)) + 1
    ny = int(np.ceil(by / el_size)) + 1
    x = np.linspace(lo[0], hi[0], nx)
    y = np.linspace(lo[1], hi[1], ny)
    X, Y = np.meshgrid(x, y)
    nn = _mgrid_numbers(ny, nx)
    e1a, e2a, e3a = nn[:-1, :-1], nn[1:, 1:], nn[1:, :-1]
    e1b, e2b, e3b = nn[:-1, :-1], nn[:-1, 1:], nn[1:, 1:]
    nds = np.column_stack([_colvec(X), _colvec(Y)])
    els = np.vstack([
        np.column_stack([_colvec(e1a), _colvec(e2a), _colvec(e3a)]),
        np.column_stack([_colvec(e1b), _colvec(e2b), _colvec(e3b)]),
    ])
    inn, out = elements_in_region(nds, els, bdry_pts)
    els = els[~out]
    nds, els, _ = remove_unused_nodes(nds, els)
    n = els.shape[0]
    return dict(nds=nds, els=els, el_mat_i=np.ones(n, np.int64), el_abs_i=np.zeros(n))


def isometric_structured_mesh(bdry_pts, el_size):
    """fn_isometric_structured_mesh.m:16-84 (equilateral triangles)."""
    bdry_pts = np.asarray(bdry_pts, float)
    lo, hi = bdry_pts.min(0), bdry_pts.max(0)
    sin60 = np.sin(np.deg2rad(60.0))
    bx = abs(hi[0] - lo[0]) + el_size
    by = abs(hi[1] - lo[1])
    nx = int(np.ceil(bx / el_size)) + 1
    ny = int(np.ceil(by / el_size / sin60)) + 1
    x = np.linspace(lo[0] - el_size / 2, hi[0] + el_size / 2, nx)
    y = np.linspace(lo[1], hi[1], ny)
    X, Y = np.meshgrid(x, y)
    X[0::2, :] += el_size / 4
    X[1::2, :] -= el_size / 4
    nn = _mgrid_numbers(ny, nx)
    fams = [
        (nn[0:-1:2, :-1], nn[1::2, 1:], nn[1::2, :-1]),
        (nn[0:-1:2, :-1], nn[0:-1:2, 1:], nn[1::2, 1:]),
        (nn[1:-1:2, 1:], nn[2::2, 1:], nn[2::2, :-1]),
        (nn[1:-1:2, :-1], nn[1:-1:2, 1:], nn[2::2, :-1]),
    ]
    blocks = [np.column_stack([_colvec(a), _colvec(b), _colvec(c)]) for a, b, c in fams]
    nds = np.column_stack([_colvec(X), _colvec(Y)])
    els = np.vstack(blocks)
    inn, out = elements_in_region(nds, els, bdry_pts)
    els = els[~out]
    nds, els, _ = remove_unused_nodes(nds, els)
    n = els.shape[0]
    return dict(nds=nds, els=els, el_mat_i=np.ones(n, np.int64))


def cubic_structured_mesh_3d(crnr_pts, el_size):
    """fn_3d_cubic_structured_mesh.m:14-46 (8-node bricks, ndgrid order)."""
    crnr_pts = np.asarray(crnr_pts, float)
    sz = crnr_pts[1] - crnr_pts[0]
    n = (np.ceil(sz / el_size) + 1).astype(np.int64)
    d = sz / (n - 1)
    I1, I2, I3 = np.meshgrid(np.arange(1, n[0] + 1), np.arange(1, n[1] + 1),
                             np.arange(1, n[2] + 1), indexing="ij")
    idx = np.column_stack([_colvec(I1), _colvec(I2), _colvec(I3)]).astype(float)
    nds = (idx - 1) * d + crnr_pts[0]
    i = np.arange(1, I1.size + 1, dtype=np.int64).reshape(tuple(n), order="F")
    els = np.column_stack([
        _colvec(i[:-1, :-1, :-1]), _colvec(i[1:, :-1, :-1]), _colvec(i[1:, 1:, :-1]),
        _colvec(i[:-1, 1:, :-1]), _colvec(i[:-1, :-1, 1:]), _colvec(i[1:, :-1, 1:]),
        _colvec(i[1:, 1:, 1:]), _colvec(i[:-1, 1:, 1:]),
    ])
    return dict(nds=nds, els=els, el_mat_i=np.ones(els.shape[0], np.int64))


def find_nodes_on_line(nds, p1, p2, tol):
    """fn_find_nodes_on_line.m:34-45; returns 1-based node list."""
    p1 = np.asarray(p1, float)
    p2 = np.asarray(p2, float)
    nvec = p2 - p1
    dd = np.sqrt(np.sum(nvec ** 2))
    nvec = nvec / dd
    s = np.sum((nds - p1) * nvec, axis=1)
    r = nds - p1 - s[:, None] * nvec
    s = s / dd
    r = np.sqrt(np.sum(r ** 2, axis=1))
    return np.nonzero((r <= tol) & (s >= 0 - tol) & (s <= 1 + tol))[0] + 1


def set_els_inside_bdry_to_mat(mod, bdry_pts, mat_i):
    """fn_set_els_inside_bdry_to_mat.m:1-10."""
    inn, _ = elements_in_region(mod["nds"], mod["els"], bdry_pts)
    mod["el_mat_i"] = np.asarray(mod["el_mat_i"]).copy()
    mod["el_mat_i"][inn] = mat_i
    return mod


def get_edges(els):
    """fn_get_edges.m:1-35: unique sorted edges and adjacent elements.

    Returns (ed, els_with_ed) where ed is (n_ed, 2) 1-based node pairs sorted
    ascending (rows sorted), and els_with_ed holds the 1-based indices of the
    adjoining elements per edge in descending order, 0-padded.
    """
    els = np.asarray(els, dtype=np.int64)
    nnz_per = (els > 0).sum(1)
    eds, eli = [], []
    # elements keep their non-zero nodes first, so edge k of an element with
    # m nodes joins columns k and (k + 1) mod m (reference :11-19)
    for m in np.unique(nnz_per):
        rows = np.nonzero(nnz_per == m)[0]
        for k in range(m):
            eds.append(np.column_stack([els[rows, k], els[rows, (k + 1) % m]]))
            eli.append(rows + 1)
    ed = np.sort(np.vstack(eds), axis=1)
    eli = np.concatenate(eli)
    order = np.lexsort((ed[:, 1], ed[:, 0]))
    ed, eli = ed[order], eli[order]
    ued, ci = np.unique(ed, axis=0, return_inverse=True)
    ci = ci.ravel()
    maxc = np.bincount(ci).max()
    ewe = np.zeros((ued.shape[0], maxc), dtype=np.int64)
    # gather elements per edge, descending
    ord2 = np.lexsort((-eli, ci))
    ci_s, el_s = ci[ord2], eli[ord2]
    start = np.searchsorted(ci_s, np.arange(ued.shape[0]))
    pos = np.arange(ci_s.size) - start[ci_s]
    ewe[ci_s, pos] = el_s
    return ued, ewe


def add_fluid_solid_interface_els(mod, matls, fluid_names=("AC2D3",),
                                  solid_names=("CPE3",), interface_name="ASI2D2"):
    """fn_add_fluid_solid_interface_els.m:1-73.

    Interface edges between fluid and solid elements become ASI2D2 elements,
    node order flipped so that the fluid element centre lies on the side of
    b = [a_y, -a_x] with a = nd2 - nd1 (reference :185-194).
    """
    nds, els = mod["nds"], np.asarray(mod["els"], dtype=np.int64)
    if "el_typ_i" not in mod:
        mod["el_typ_i"] = [matls[m - 1]["el_typ"] for m in mod["el_mat_i"]]
    typ = np.array(list(mod["el_typ_i"]), dtype=object)
    ed, ewe = get_edges(els)
    invalid = ewe == 0
    idx = np.where(invalid, 1, ewe) - 1
    et = typ[idx]
    et[invalid] = ""
    fl = np.isin(et, fluid_names)
    so = np.isin(et, solid_names)
    if et.shape[1] < 2:
        j = np.zeros(ed.shape[0], bool)
    else:
        j = (fl[:, 0] & so[:, 1]) | (fl[:, 1] & so[:, 0])
    et, ewe, ed = et[j], ewe[j], ed[j].copy()
    for i in range(ed.shape[0]):
        e = ewe[i][np.isin(et[i], fluid_names)]
        ec = calc_element_centres(nds, els[e - 1])[0]
        a = nds[ed[i, 1] - 1] - nds[ed[i, 0] - 1]
        b = np.array([a[1], -a[0]])
        c = ec - nds[ed[i, 0] - 1]
        if np.dot(c, b) < 0:
            ed[i] = ed[i, ::-1]
    nint = ed.shape[0]
    pad = np.zeros((nint, els.shape[1] - 2), dtype=np.int64)
    mod["els"] = np.vstack([els, np.hstack([ed, pad])])
    mod["el_typ_i"] = list(mod["el_typ_i"]) + [interface_name] * nint
    mod["el_mat_i"] = np.concatenate([np.asarray(mod["el_mat_i"]), np.zeros(nint, np.int64)])
    if "el_abs_i" in mod:
        mod["el_abs_i"] = np.concatenate([np.asarray(mod["el_abs_i"], float), np.zeros(nint)])
    return mod


def dist_point_to_bdry_2d(pts, bdry):
    """fn_dist_point_to_bdry_2D.m:1-69 (nearest vertex and its two edges)."""
    pts = np.asarray(pts, float)
    bdry = np.asarray(bdry, float)
    nb = bdry.shape[0]
    r0all = np.sqrt(((pts[:, None, :] - bdry[None, :, :]) ** 2).sum(-1))
    j = np.argmin(r0all, axis=1)           # first minimum, like MATLAB min
    r0 = r0all[np.arange(pts.shape[0]), j]
    j1 = (j + 1) % nb
    j2 = (j - 1) % nb

    def dist_line(p, a, b):
        nvec = b - a
        dd = np.sqrt((nvec ** 2).sum(-1, keepdims=True))
        nvec = nvec / dd
        s = ((p - a) * nvec).sum(-1, keepdims=True)
        r = p - a - s * nvec
        s = s / dd
        return np.sqrt((r ** 2).sum(-1)), s[:, 0]

    r1, s1 = dist_line(pts, bdry[j], bdry[j1])
    r1 = np.where((s1 < 0) | (s1 > 1), np.inf, r1)
    r2, s2 = dist_line(pts, bdry[j], bdry[j2])
    r2 = np.where((s2 < 0) | (s2 > 1), np.inf, r2)
    return np.minimum(np.minimum(r0, r1), r2)


def add_absorbing_layer(mod, abs_bdry_pts, abs_bdry_thickness):
    """fn_add_absorbing_layer.m:1-17."""
    ctr = calc_element_centres(mod["nds"], mod["els"])
    d = dist_point_to_bdry_2d(ctr, abs_bdry_pts)
    inn = inpolygon(ctr[:, 0], ctr[:, 1], abs_bdry_pts)
    a = d / abs_bdry_thickness
    a = np.clip(a, 0.0, 1.0)
    a[inn] = 0.0
    mod["el_abs_i"] = a
    return mod


def create_smooth_random_blob(min_rad_frac, complexity, no_pts, rng):
    """fn_create_smooth_random_blob.m:1-14 with a seeded generator."""
    a = np.linspace(0, 2 * np.pi, no_pts + 1)[:-1]
    if complexity > 0:
        n = np.arange(0, complexity + 1)
        phi = rng.random(n.size) * 2 * np.pi
        r = np.sin(a[:, None] * n[None, :] + phi[None, :]).sum(1)
        r = (r - r.min()) / (r.max() - r.min()) * (1 - min_rad_frac) + min_rad_frac
    else:
        r = np.ones_like(a)
    return r[:, None] * np.column_stack([np.cos(a), np.sin(a)])


def remove_elements_in_region(mod, region):
    """Void scatterer: fn_add_scatterer.m:16-20 with scat_matl = 0."""
    inn, _ = elements_in_region(mod["nds"], mod["els"], region)
    keep = ~inn
    for k in ("els", "el_mat_i", "el_abs_i"):
        if k in mod:
            mod[k] = np.asarray(mod[k])[keep]
    if "el_typ_i" in mod:
        mod["el_typ_i"] = [t for t, k in zip(mod["el_typ_i"], keep) if k]
    mod["nds"], mod["els"], _ = remove_unused_nodes(mod["nds"], mod["els"])
    return mod
