"""Synthetic MPAS cases: icosahedral Voronoi meshes and analytic dry initial states.

The reference ships no meshes or initial conditions (it expects MPAS
``init_atmosphere`` output fetched over the network), so this module builds the
raw grid/init arrays that an MPAS ``x1.N.grid.nc`` / ``x1.N.init.nc`` pair would
hold, in the same raw layout the reference loader reads
(``mpas_pytorch/ic_loader.py:138-176``): unpadded arrays, 1-based connectivity,
Fortran dimension order reversed (``(nEdges, 2)``, ``(nCells, nVertLevels)`` ...).

Mesh: an icosahedron refined ``level`` times by edge bisection (C = 10*4**level + 2
generators) and its spherical Voronoi dual (vertices = triangle circumcentres).
Conventions follow the MPAS mesh specification:

* ``cellsOnEdge = (c1, c2)``; the edge normal points from c1 to c2.
* ``verticesOnEdge = (v1, v2)``; the tangent ``t = k x n`` points from v1 to v2.
* ``cellsOnCell/edgesOnCell`` are counter-clockwise (seen from outside);
  ``verticesOnCell[i]`` lies between ``edgesOnCell[i]`` and ``edgesOnCell[i+1]``.
* ``weightsOnEdge/edgesOnEdge`` are the TRiSK tangential-reconstruction weights
  (Thuburn et al. 2009, Ringler et al. 2010) with the ``dvEdge/dcEdge`` factor folded in,
  so that ``v_e = sum_j weightsOnEdge[e, j] * u[edgesOnEdge[e, j]]``.
* ``deriv_two`` holds, for each side of an edge, least-squares second-derivative
  weights along the edge normal (cell itself first, then ``cellsOnCell`` order), the
  input the reference turns into ``adv_coefs`` (``ic_loader.py:358-452``).
* ``defc_a/defc_b`` are the Smagorinsky deformation weights from Gauss' theorem.

Vertical: height coordinate over a flat surface, so ``zz = 1`` and
``zb = zb3 = zxu = 0``; MPAS vertical metrics (``rdzw, rdzu, fzm, fzp, cf1..cf3``).  With
``CaseSpec.terrain`` > 0, terrain-following levels over a cosine hill
(``zgrid = zw + h (1 - zw / ztop)``) with the metric terms ``zz``, ``zxu``, ``zb``, ``zb3``
of MPAS init, and every profile evaluated at each layer's own height.

State: dry; ``theta = 300 K exp(N^2 z / g)``; zonal ``u = 20 cos(lat)``; hydrostatic
Exner with a latitude-dependent surface value for gradient-wind balance of the
solid-body flow; seeded Gaussian theta bumps (radius 500 km, amplitude U[-1, 1] K,
sine vertical envelope) applied at constant pressure (rho*theta held fixed).
Passive tracers (cosine bell, slotted cylinder, smooth product field, all in [0, 1])
fill ``scalars`` with ``moist_end = 0`` so the run stays dry.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import detmath as dm

EARTH_RADIUS = 6371229.0
OMEGA = 7.29212e-5
GRAVITY = 9.80616
RGAS = 287.0
CP = 1004.5
P0 = 100000.0


# --------------------------------------------------------------------------------------
# icosphere
# --------------------------------------------------------------------------------------

def _icosahedron():
    t = (1.0 + math.sqrt(5.0)) / 2.0
    p = np.array(
        [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
         [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
         [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    f = np.array(
        [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
         [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
         [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
         [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    p = _unit(p)
    # orient every face counter-clockwise seen from outside
    a, b, c = p[f[:, 0]], p[f[:, 1]], p[f[:, 2]]
    flip = _dot(_cross(b - a, c - a), a + b + c) < 0
    f[flip] = f[flip][:, [0, 2, 1]]
    return p, f


def icosphere(level: int):
    """Unit-sphere generators and CCW triangles of a ``level``-times bisected icosahedron."""
    p, f = _icosahedron()
    for _ in range(level):
        n = p.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        key = np.minimum(e[:, 0], e[:, 1]) * (n + 1) + np.maximum(e[:, 0], e[:, 1])
        uniq, inv = np.unique(key, return_inverse=True)
        lo = uniq // (n + 1)
        hi = uniq % (n + 1)
        mid = _unit(p[lo] + p[hi])
        mid_id = n + inv
        nf = f.shape[0]
        ab, bc, ca = mid_id[:nf], mid_id[nf:2 * nf], mid_id[2 * nf:]
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        f = np.concatenate([
            np.stack([a, ab, ca], 1), np.stack([ab, b, bc], 1),
            np.stack([ca, bc, c], 1), np.stack([ab, bc, ca], 1)])
        p = np.concatenate([p, mid])
    return p, f


# Vector algebra written out component by component (fixed evaluation order), and the
# elementary functions of detmath: the generated arrays are bit-identical on every machine.

def _dot(a, b):
    return a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1] + a[..., 2] * b[..., 2]


def _cross(a, b):
    return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1],
                     a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                     a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], -1)


def _norm(v):
    return np.sqrt(_dot(v, v))


def _unit(v):
    return v / _norm(v)[..., None]


def _arc(a, b):
    """Great-circle angle between unit vectors (robust atan2 form)."""
    return dm.atan2(_norm(_cross(a, b)), _dot(a, b))


def _sph_tri_area(a, b, c):
    """Spherical-excess area of unit-sphere triangles (Eriksson's formula)."""
    num = np.abs(_dot(a, _cross(b, c)))
    den = 1.0 + _dot(a, b) + _dot(b, c) + _dot(c, a)
    return 2.0 * dm.atan2(num, den)


def _latlon(x):
    lat = dm.asin(np.clip(x[:, 2], -1.0, 1.0))
    lon = np.mod(dm.atan2(x[:, 1], x[:, 0]), 2.0 * math.pi)
    return lat, lon


def _east_north(x):
    """Local east and north unit vectors at unit positions ``x``."""
    k = np.array([0.0, 0.0, 1.0])
    east = _cross(k, x)
    nrm = _norm(east)[..., None]
    east = np.where(nrm > 1e-14, east / np.maximum(nrm, 1e-300), np.array([0.0, 1.0, 0.0]))
    north = _cross(x, east)
    return east, north


def _lsq_xx_weights(px, py, valid):
    """Weights ``w`` (n, m) such that ``sum_j w[:, j] f_j`` is the second derivative in x
    at the origin of the least-squares quadratic ``a0 + a1 x + a2 y + a3 x^2 + a4 xy +
    a5 y^2`` through the valid points ``(px, py)``: twice row 3 of the fit's pseudo-inverse.
    Normal equations in coordinates scaled by the stencil's extent, Cholesky factor, one
    solve for row 3 of the inverse."""
    n, m = px.shape
    h = np.max(np.where(valid, np.maximum(np.abs(px), np.abs(py)), 0.0), axis=1)
    xs, ys = px / h[:, None], py / h[:, None]
    B = np.stack([np.ones_like(xs), xs, ys, xs * xs, xs * ys, ys * ys], -1) * valid[..., None]
    N = np.zeros((n, 6, 6))
    for i in range(6):
        for j in range(i + 1):
            s = B[:, 0, i] * B[:, 0, j]
            for r in range(1, m):
                s = s + B[:, r, i] * B[:, r, j]
            N[:, i, j] = N[:, j, i] = s
    L = np.zeros((n, 6, 6))
    for j in range(6):
        d = N[:, j, j]
        for k in range(j):
            d = d - L[:, j, k] * L[:, j, k]
        L[:, j, j] = np.sqrt(d)
        for i in range(j + 1, 6):
            s = N[:, i, j]
            for k in range(j):
                s = s - L[:, i, k] * L[:, j, k]
            L[:, i, j] = s / L[:, j, j]
    y = np.zeros((n, 6))   # L y = e_3
    for i in range(6):
        s = np.full(n, 1.0 if i == 3 else 0.0)
        for k in range(i):
            s = s - L[:, i, k] * y[:, k]
        y[:, i] = s / L[:, i, i]
    z = np.zeros((n, 6))   # L^T z = y: z = N^-1 e_3
    for i in reversed(range(6)):
        s = y[:, i]
        for k in range(i + 1, 6):
            s = s - L[:, k, i] * z[:, k]
        z[:, i] = s / L[:, i, i]
    w = B[..., 0] * z[:, None, 0]
    for i in range(1, 6):
        w = w + B[..., i] * z[:, None, i]
    return 2.0 * w / (h * h)[:, None]


# --------------------------------------------------------------------------------------
# Voronoi mesh with MPAS connectivity and geometry
# --------------------------------------------------------------------------------------

def build_mesh(level: int, radius: float = EARTH_RADIUS) -> dict:
    """Raw MPAS grid arrays (unpadded, 1-based connectivity) for an icosahedral mesh."""
    pc, tri = icosphere(level)
    nc = pc.shape[0]
    nv = tri.shape[0]

    # Voronoi vertices: circumcentres of the CCW triangles
    a, b, c = pc[tri[:, 0]], pc[tri[:, 1]], pc[tri[:, 2]]
    pv = _unit(_cross(b - a, c - a))

    # directed half-edges of every triangle: (from, to, face); face lies left of from->to
    h_from = np.concatenate([tri[:, 0], tri[:, 1], tri[:, 2]])
    h_to = np.concatenate([tri[:, 1], tri[:, 2], tri[:, 0]])
    h_face = np.concatenate([np.arange(nv)] * 3)
    h_third = np.concatenate([tri[:, 2], tri[:, 0], tri[:, 1]])

    # undirected edges, c1 = lower index
    lo = np.minimum(h_from, h_to)
    hi = np.maximum(h_from, h_to)
    key = lo * nc + hi
    uniq, inv = np.unique(key, return_inverse=True)
    ne = uniq.shape[0]
    c1 = uniq // nc
    c2 = uniq % nc
    # v2 = face with directed half-edge c1 -> c2 (left of the normal), v1 = the other
    fwd = h_from == lo
    v2 = np.empty(ne, np.int64)
    v1 = np.empty(ne, np.int64)
    v2[inv[fwd]] = h_face[fwd]
    v1[inv[~fwd]] = h_face[~fwd]

    # per-cell CCW neighbour rings from the half-edges (from=centre, to=x, third=y:
    # around the centre, x is followed counter-clockwise by y)
    order = np.argsort(h_from, kind="stable")
    cen = h_from[order]
    xs = h_to[order]
    ys = h_third[order]
    fs = h_face[order]
    counts = np.bincount(cen, minlength=nc)
    maxe = int(counts.max())
    start = np.concatenate([[0], np.cumsum(counts)[:-1]])
    slot = np.arange(cen.shape[0]) - start[cen]
    X = np.full((nc, maxe), -1, np.int64)
    Y = np.full((nc, maxe), -2, np.int64)
    F = np.full((nc, maxe), -1, np.int64)
    X[cen, slot] = xs
    Y[cen, slot] = ys
    F[cen, slot] = fs
    succ = np.argmax(X[:, None, :] == Y[:, :, None], axis=2)  # slot whose x == my y
    ring = np.zeros((nc, maxe), np.int64)
    cur = np.zeros(nc, np.int64)
    rows = np.arange(nc)
    for k in range(maxe):
        ring[:, k] = cur
        cur = succ[rows, cur]
    cells_on_cell = np.where(np.arange(maxe)[None, :] < counts[:, None], X[rows[:, None], ring], -1)
    verts_on_cell = np.where(np.arange(maxe)[None, :] < counts[:, None], F[rows[:, None], ring], -1)
    # rotate each ring so it starts at its lowest-index neighbour (deterministic)
    big = np.where(cells_on_cell >= 0, cells_on_cell, np.iinfo(np.int64).max)
    s0 = np.argmin(big, axis=1)
    idx = (s0[:, None] + np.arange(maxe)[None, :]) % counts[:, None]
    cells_on_cell = np.where(np.arange(maxe)[None, :] < counts[:, None], cells_on_cell[rows[:, None], idx], -1)
    verts_on_cell = np.where(np.arange(maxe)[None, :] < counts[:, None], verts_on_cell[rows[:, None], idx], -1)

    def edge_id(p, q):
        kk = np.minimum(p, q) * nc + np.maximum(p, q)
        return np.searchsorted(uniq, kk)

    valid = cells_on_cell >= 0
    edges_on_cell = np.where(valid, edge_id(np.repeat(rows[:, None], maxe, 1), np.where(valid, cells_on_cell, 0)), -1)

    # vertices: CCW cells (triangle order), edgesOnVertex[i] between cell i and i+1
    cells_on_vertex = tri.copy()
    edges_on_vertex = np.stack([edge_id(tri[:, 0], tri[:, 1]), edge_id(tri[:, 1], tri[:, 2]),
                                edge_id(tri[:, 2], tri[:, 0])], 1)

    # geometry
    pe = _unit(pc[c1] + pc[c2])
    dc = radius * _arc(pc[c1], pc[c2])
    dv = radius * _arc(pv[v1], pv[v2])
    # kites: cell i of vertex v = quad (cell, edge(i,i-1) midpoint, vertex, edge(i,i+1) midpoint)
    kites = np.zeros((nv, 3))
    for i in range(3):
        cc = pc[tri[:, i]]
        e_next = pe[edges_on_vertex[:, i]]
        e_prev = pe[edges_on_vertex[:, (i + 2) % 3]]
        kites[:, i] = _sph_tri_area(cc, e_prev, pv) + _sph_tri_area(cc, pv, e_next)
    kites *= radius * radius
    area_tri = (radius * radius) * _sph_tri_area(a, b, c)
    area_cell = np.zeros(nc)
    for i in range(3):
        np.add.at(area_cell, tri[:, i], kites[:, i])

    latc, lonc = _latlon(pc)
    late, lone = _latlon(pe)
    latv, lonv = _latlon(pv)
    nvec = _unit(pc[c2] - pc[c1] - _dot(pc[c2] - pc[c1], pe)[:, None] * pe)
    east_e, north_e = _east_north(pe)
    angle_edge = dm.atan2(_dot(nvec, north_e), _dot(nvec, east_e))

    # kite area of cell `cell` at vertex `vtx`
    def kite_of(cell, vtx):
        m = cells_on_vertex[vtx] == cell[..., None]
        k = np.where(m, kites[vtx], 0.0)
        return k[..., 0] + k[..., 1] + k[..., 2]

    # ---- TRiSK weights ----------------------------------------------------------
    n_eoe = counts[c1] + counts[c2] - 2
    max2 = 2 * maxe
    eoe = np.zeros((ne, max2), np.int64) - 1
    woe = np.zeros((ne, max2))
    eids = np.arange(ne)
    col = np.zeros(ne, np.int64)
    for side, cell, sgn in ((0, c1, 1.0), (1, c2, -1.0)):
        n = counts[cell]
        eoc = edges_on_cell[cell]
        voc = verts_on_cell[cell]
        pos = np.argmax(eoc == eids[:, None], axis=1)
        r = np.zeros(ne)
        for j in range(1, maxe):
            act = j < n
            k = (pos + j) % n
            kprev = (pos + j - 1) % n
            e2 = eoc[eids, k]
            vtx = voc[eids, kprev]  # vertex between the previous edge and e2
            r = r + np.where(act, kite_of(cell, np.where(act, vtx, 0)) / area_cell[cell], 0.0)
            # orientation of e2 relative to `cell`: +1 if its normal points out of `cell`
            out = np.where(c1[np.where(act, e2, 0)] == cell, 1.0, -1.0)
            w = sgn * (0.5 - r) * out * dv[np.where(act, e2, 0)] / dc
            eoe[eids[act], col[act]] = e2[act]
            woe[eids[act], col[act]] = w[act]
            col = col + act
    assert np.all(col == n_eoe)

    # ---- deriv_two: LSQ second derivative along the edge normal -----------------------
    deriv_two = np.zeros((ne, 2, 15))
    for side, cell in ((0, c1), (1, c2)):
        n = counts[cell]
        pts = np.concatenate([cell[:, None], np.where(cells_on_cell[cell] >= 0, cells_on_cell[cell], cell[:, None])], 1)
        pts_valid = np.concatenate([np.ones((ne, 1), bool), cells_on_cell[cell] >= 0], 1)
        x0 = pc[cell]
        xh = nvec - _dot(nvec, x0)[:, None] * x0
        xh = _unit(xh)
        yh = _cross(x0, xh)
        q = pc[pts]  # (ne, 7, 3)
        # gnomonic-style local coordinates scaled by arc length
        d = q - x0[:, None, :]
        px = radius * _dot(d, xh[:, None, :])
        py = radius * _dot(d, yh[:, None, :])
        deriv_two[:, side, : maxe + 1] = _lsq_xx_weights(px, py, pts_valid) * pts_valid

    # ---- Smagorinsky deformation weights ---------------------------------------------
    defc_a = np.zeros((nc, maxe))
    defc_b = np.zeros((nc, maxe))
    east_c, north_c = _east_north(pc)
    for i in range(maxe):
        act = i < counts
        e = np.where(act, edges_on_cell[:, i], 0)
        s = np.where(c1[e] == rows, 1.0, -1.0)
        nn = nvec[e]
        th = dm.atan2(_dot(nn, north_c), _dot(nn, east_c))
        defc_a[:, i] = np.where(act, s * dv[e] * dm.cos(2.0 * th) / area_cell, 0.0)
        defc_b[:, i] = np.where(act, s * dv[e] * dm.sin(2.0 * th) / area_cell, 0.0)

    one = lambda x: (x + 1).astype(np.int32)
    zero_pad = lambda x: np.where(x >= 0, x + 1, 0).astype(np.int32)
    mesh = {
        "nCells": nc, "nEdges": ne, "nVertices": nv, "maxEdges": maxe, "maxEdges2": max2,
        "vertexDegree": 3,
        "cellsOnCell": zero_pad(cells_on_cell),
        "edgesOnCell": zero_pad(edges_on_cell),
        "verticesOnCell": zero_pad(verts_on_cell),
        "nEdgesOnCell": counts.astype(np.int32),
        "cellsOnEdge": one(np.stack([c1, c2], 1)),
        "verticesOnEdge": one(np.stack([v1, v2], 1)),
        "edgesOnVertex": one(edges_on_vertex),
        "cellsOnVertex": one(cells_on_vertex),
        "edgesOnEdge": zero_pad(eoe),
        "nEdgesOnEdge": n_eoe.astype(np.int32),
        "weightsOnEdge": woe,
        "dcEdge": dc, "dvEdge": dv,
        "kiteAreasOnVertex": kites, "areaCell": area_cell, "areaTriangle": area_tri,
        "latCell": latc, "lonCell": lonc, "latEdge": late, "lonEdge": lone,
        "latVertex": latv, "lonVertex": lonv,
        "xCell": radius * pc[:, 0], "yCell": radius * pc[:, 1], "zCell": radius * pc[:, 2],
        "xEdge": radius * pe[:, 0], "yEdge": radius * pe[:, 1], "zEdge": radius * pe[:, 2],
        "xVertex": radius * pv[:, 0], "yVertex": radius * pv[:, 1], "zVertex": radius * pv[:, 2],
        "angleEdge": angle_edge,
        "fEdge": 2.0 * OMEGA * dm.sin(late), "fVertex": 2.0 * OMEGA * dm.sin(latv),
        "meshDensity": np.ones(nc),
        "indexToCellID": np.arange(1, nc + 1, dtype=np.int32),
        "indexToEdgeID": np.arange(1, ne + 1, dtype=np.int32),
        "indexToVertexID": np.arange(1, nv + 1, dtype=np.int32),
        "deriv_two": deriv_two,
        "defc_a": defc_a, "defc_b": defc_b,
        "on_a_sphere": 1,
    }
    return mesh


# --------------------------------------------------------------------------------------
# vertical grid and analytic state
# --------------------------------------------------------------------------------------

def vertical_levels(nlev: int, ztop: float = 30000.0, dz_bottom: float | None = None) -> np.ndarray:
    """W-level heights ``zw[0..nlev]``: uniform, or geometrically stretched from ``dz_bottom``."""
    if dz_bottom is None:
        return np.linspace(0.0, ztop, nlev + 1)
    # find growth ratio q with dz_bottom * (q**nlev - 1)/(q - 1) = ztop
    def powers(q):  # q**0 .. q**nlev by repeated multiplication (no libm pow)
        out = [1.0]
        for _ in range(nlev):
            out.append(out[-1] * q)
        return np.array(out)

    lo_q, hi_q = 1.0 + 1e-12, 2.0
    for _ in range(200):
        q = 0.5 * (lo_q + hi_q)
        tot = dz_bottom * (powers(q)[nlev] - 1.0) / (q - 1.0)
        if tot > ztop:
            hi_q = q
        else:
            lo_q = q
    dz = dz_bottom * powers(q)[:nlev]
    zw = np.concatenate([[0.0], np.cumsum(dz)])
    zw *= ztop / zw[-1]
    return zw


@dataclass(frozen=True)
class CaseSpec:
    """One synthetic case: mesh level, vertical grid, perturbations and tracers."""

    level: int = 4
    nlev: int = 26
    ztop: float = 30000.0
    dz_bottom: float | None = None
    seed: int = 0
    n_bumps: int = 8
    n_tracers: int = 1
    u_noise: float = 0.0
    w_sine: float = 0.0
    round_wind_bits: int = 0
    qv_surface: float = 0.0  # > 0: moist case, water vapour as scalar 0 (moist_end = 1)
    uv_init: tuple = (0.0, 0.0)  # initial (u, v) profile values (read by config_mix_full = false)
    terrain: float = 0.0  # > 0: peak height (m) of a cosine-hill mountain, terrain-following levels


def _vertical_metrics(zw: np.ndarray) -> dict:
    nz = zw.shape[0]
    nz1 = nz - 1
    dzw = zw[1:] - zw[:-1]
    rdzw = 1.0 / dzw
    dzu = np.zeros(nz1)
    rdzu = np.zeros(nz1)
    fzm = np.zeros(nz1)
    fzp = np.zeros(nz1)
    for k in range(1, nz1):
        dzu[k] = 0.5 * (dzw[k] + dzw[k - 1])
        rdzu[k] = 1.0 / dzu[k]
        fzp[k] = 0.5 * dzw[k] / dzu[k]
        fzm[k] = 0.5 * dzw[k - 1] / dzu[k]
    d1 = 0.5 * dzw[0]
    d2 = dzw[0] + 0.5 * dzw[1]
    d3 = dzw[0] + dzw[1] + 0.5 * dzw[2]
    den = d2 * d3 * (d3 - d2) + d1 * d3 * (d1 - d3) + d1 * d2 * (d2 - d1)
    cf1 = d2 * d3 * (d3 - d2) / den
    cf2 = d1 * d3 * (d1 - d3) / den
    cf3 = d1 * d2 * (d2 - d1) / den
    return {
        "rdzw": rdzw, "dzw": dzw, "rdzu": rdzu, "dzu": dzu, "fzm": fzm, "fzp": fzp,
        "fnm": fzm.copy(), "fnp": fzp.copy(), "rdnw": rdzw.copy(),
        "cf1": np.float64(cf1), "cf2": np.float64(cf2), "cf3": np.float64(cf3),
    }


def _exner_profile(zmid: np.ndarray, theta0: float, bvf: float, pi_s: np.ndarray) -> np.ndarray:
    """Hydrostatic Exner for theta = theta0 exp(N^2 z/g): d(pi)/dz = -g/(cp theta); zmid the
    layer heights, one profile (nlev) or per cell (nc, nlev)."""
    g = GRAVITY
    z = zmid[None, :] if zmid.ndim == 1 else zmid
    return pi_s[:, None] - g * g / (CP * theta0 * bvf * bvf) * (1.0 - dm.exp(-bvf * bvf * z / g))


def _terrain_height(mesh: dict, spec: "CaseSpec", radius: float) -> np.ndarray:
    """Surface height per cell: a cosine hill of peak ``spec.terrain`` and radius 3000 km
    centred at (lon, lat) = (90 E, 30 N)."""
    lat0, lon0 = math.pi / 6, math.pi / 2
    cl0 = float(dm.cos(lat0))
    cen = np.array([cl0 * float(dm.cos(lon0)), cl0 * float(dm.sin(lon0)), float(dm.sin(lat0))])
    pc = np.stack([mesh["xCell"], mesh["yCell"], mesh["zCell"]], 1) / radius
    r = radius * _arc(pc, cen[None, :]) / 3.0e6
    return np.where(r < 1.0, spec.terrain * 0.5 * (1.0 + dm.cos(math.pi * r)), 0.0)


def _terrain_metrics(mesh: dict, zw: np.ndarray, zgrid: np.ndarray, deriv_two: np.ndarray) -> dict:
    """Metric terms of terrain-following levels zgrid (C, L+1) over the flat levels zw, as
    MPAS init writes them: zz = dzw / dz per layer; the edge slope of each w level
    zx = (z_2 - z_1) / dcEdge and its layer mean zxu; zb, the level's height at the edge
    relative to each cell, (z_edge - z_cell) dvEdge / areaCell; zb3, its third-order
    correction -(dcEdge^2 / 12) mean(d2z/dx2 of the two cells) dvEdge / areaCell, the
    second derivatives from deriv_two (cell itself, then cellsOnCell)."""
    nc, ne = mesh["nCells"], mesh["nEdges"]
    c1 = mesh["cellsOnEdge"][:, 0] - 1
    c2 = mesh["cellsOnEdge"][:, 1] - 1
    dc, dv, area = mesh["dcEdge"], mesh["dvEdge"], mesh["areaCell"]
    zz = (zw[1:] - zw[:-1])[None, :] / (zgrid[:, 1:] - zgrid[:, :-1])
    zx = (zgrid[c2] - zgrid[c1]) / dc[:, None]
    zxu = 0.5 * (zx[:, 1:] + zx[:, :-1])
    coc = mesh["cellsOnCell"].astype(np.int64) - 1
    d2 = []
    for side, cell in ((0, c1), (1, c2)):
        nb = coc[cell]  # (ne, maxe), -1 where empty
        acc = deriv_two[:, side, 0][:, None] * zgrid[cell]
        for j in range(nb.shape[1]):
            ok = nb[:, j] >= 0
            acc = acc + np.where(ok, deriv_two[:, side, j + 1], 0.0)[:, None] * zgrid[np.where(ok, nb[:, j], cell)]
        d2.append(acc)
    z_edge = 0.5 * (zgrid[c1] + zgrid[c2])
    z_edge3 = -(dc * dc / 12.0)[:, None] * (0.5 * (d2[0] + d2[1]))
    zb = np.stack([(z_edge - zgrid[c1]) * (dv / area[c1])[:, None],
                   (z_edge - zgrid[c2]) * (dv / area[c2])[:, None]], 1)
    zb3 = np.stack([z_edge3 * (dv / area[c1])[:, None], z_edge3 * (dv / area[c2])[:, None]], 1)
    return {"zz": zz, "zxu": zxu, "zb": zb, "zb3": zb3}


def _random_direction(rng) -> np.ndarray:
    """A uniformly distributed unit vector: uniform points of the cube kept inside the unit
    ball, normalised (uniform draws and basic arithmetic only)."""
    while True:
        v = 2.0 * rng.random(3) - 1.0
        r2 = float(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
        if 1e-6 < r2 <= 1.0:
            return v / math.sqrt(r2)


def _normal(rng, shape) -> np.ndarray:
    """Standard normal draws by the Box-Muller transform of uniform draws."""
    u1 = 1.0 - rng.random(shape)  # (0, 1]
    u2 = rng.random(shape)
    return np.sqrt(-2.0 * dm.log(u1)) * dm.cos((2.0 * math.pi) * u2)


def damping_coefficients(zgrid: np.ndarray, zd: float = 22000.0, xnutr: float = 0.2) -> np.ndarray:
    """Rayleigh damping of w above ``zd`` as MPAS init computes it (the reference's
    initialization.py:333 compute_damping_coefs, mesh density 1): xnutr sin^2(pi/2 (z -
    zd) / (ztop - zd)) at the layer midpoints above zd, 0 below.  Written into the case's
    initial-condition arrays so that every loader takes these values as they are."""
    nlev = zgrid.shape[1] - 1
    zt = zgrid[:, nlev]
    zmid = 0.5 * (zgrid[:, :nlev] + zgrid[:, 1:])
    arg = 0.5 * math.pi * (zmid - zd) / (zt[:, None] - zd)
    s = dm.sin(arg)
    return np.where(zmid > zd, xnutr * (s * s), 0.0)


def initial_state(mesh: dict, spec: CaseSpec, radius: float = EARTH_RADIUS) -> dict:
    """Raw init arrays for ``spec`` on ``mesh`` (unpadded, MPAS raw layout)."""
    rng = np.random.default_rng(spec.seed)
    nc, ne = mesh["nCells"], mesh["nEdges"]
    zw = vertical_levels(spec.nlev, spec.ztop, spec.dz_bottom)
    vm = _vertical_metrics(zw)
    nlev = spec.nlev
    zmid = 0.5 * (zw[1:] + zw[:-1])
    theta0, bvf, u0 = 300.0, 0.01, 20.0
    latc = mesh["latCell"]
    # terrain-following levels over a mountain: every profile at the layer's own height
    hill = _terrain_height(mesh, spec, radius) if spec.terrain > 0.0 else None
    if hill is not None:
        zgrid = zw[None, :] + hill[:, None] * (1.0 - zw[None, :] / spec.ztop)
        zmid = 0.5 * (zgrid[:, 1:] + zgrid[:, :-1])  # (nc, nlev)

    # surface Exner balancing the solid-body zonal flow u0 cos(lat) (gradient wind)
    sl = dm.sin(latc)
    pi_s = 1.0 - (u0 * (2.0 * OMEGA * radius + u0) * 0.5 * (sl * sl)) / (CP * theta0)
    if hill is None:
        theta_b = theta0 * dm.exp(bvf * bvf * zmid / GRAVITY)[None, :].repeat(nc, 0)
    else:
        theta_b = theta0 * dm.exp(bvf * bvf * zmid / GRAVITY)
    exner_b = _exner_profile(zmid, theta0, bvf, pi_s)
    p_b = P0 * dm.pow(exner_b, CP / RGAS)
    rho_b = p_b / (RGAS * theta_b * exner_b)

    # theta bumps at constant pressure (rho*theta fixed)
    pc = np.stack([mesh["xCell"], mesh["yCell"], mesh["zCell"]], 1) / radius
    theta = theta_b.copy()
    env = dm.sin(math.pi * zmid / spec.ztop)
    env = env[None, :] if env.ndim == 1 else env
    for _ in range(spec.n_bumps):
        v = _random_direction(rng)
        amp = rng.uniform(-1.0, 1.0)
        dist = radius * _arc(pc, v[None, :])
        r = dist / 500.0e3
        theta += amp * dm.exp(-(r * r))[:, None] * env
    rho = rho_b * theta_b / theta

    # edge winds
    pe = np.stack([mesh["xEdge"], mesh["yEdge"], mesh["zEdge"]], 1) / radius
    c1 = mesh["cellsOnEdge"][:, 0] - 1
    c2 = mesh["cellsOnEdge"][:, 1] - 1
    nvec = pc[c2] - pc[c1]
    nvec = _unit(nvec - _dot(nvec, pe)[:, None] * pe)
    east_e, _ = _east_north(pe)
    un = u0 * dm.cos(mesh["latEdge"]) * _dot(east_e, nvec)
    u = np.repeat(un[:, None], nlev, 1)
    if spec.u_noise > 0.0:
        u = u + spec.u_noise * _normal(rng, u.shape)
    if spec.round_wind_bits > 0:
        m, e = np.frexp(u)
        scale = float(2 ** spec.round_wind_bits)
        u = np.ldexp(np.round(m * scale) / scale, e)

    w = np.zeros((nc, nlev + 1))
    if spec.w_sine != 0.0:
        lonc = mesh["lonCell"]
        w[:, 1:nlev] = spec.w_sine * dm.sin(math.pi * zw[None, 1:nlev] / spec.ztop) * dm.cos(latc)[:, None] \
            * dm.sin(2.0 * lonc)[:, None]

    # passive tracers in [0, 1]
    lonc = mesh["lonCell"]
    tracers = []
    for t in range(spec.n_tracers):
        kind = t % 3
        if kind == 0:  # cosine bell centred at (lon, lat) = (3pi/2, 0)
            r = _arc(pc, np.array([0.0, -1.0, 0.0])[None, :])
            h = np.where(r < 0.5, 0.5 * (1.0 + dm.cos(math.pi * r / 0.5)), 0.0)
        elif kind == 1:  # slotted cylinder centred at (lon, lat) = (pi/2, pi/6)
            cen = np.array([0.0, float(dm.cos(math.pi / 6)), float(dm.sin(math.pi / 6))])
            r = _arc(pc, cen[None, :])
            dlon = lonc - math.pi / 2
            dlon = dlon - (2.0 * math.pi) * np.rint(dlon / (2.0 * math.pi))  # wrapped to [-pi, pi]
            slot = (np.abs(dlon) < 1.0 / 12.0) & (latc < math.pi / 6 + 5.0 / 24.0)
            h = np.where((r < 0.5) & ~slot, 1.0, 0.1)
        else:  # smooth product field
            cl = dm.cos(latc)
            h = 0.5 + 0.5 * (cl * cl) * dm.cos(2.0 * lonc)
        tracers.append(np.repeat(h[:, None], nlev, 1))
    qv = np.zeros((nc, nlev))
    if spec.qv_surface > 0.0:  # vapour decaying with a 2.5 km scale height, wetter at the equator
        cl = dm.cos(latc)
        decay = dm.exp(-zmid / 2500.0)
        qv = spec.qv_surface * (decay[None, :] if decay.ndim == 1 else decay) * (0.25 + 0.75 * (cl * cl))[:, None]
        tracers = [qv] + tracers
    scalars = np.stack(tracers, -1) if tracers else np.zeros((nc, nlev, 0))

    if hill is None:
        zgrid = np.repeat(zw[None, :], nc, 0)
        metrics = {"zz": np.ones((nc, nlev)), "zb": np.zeros((ne, 2, nlev + 1)),
                   "zb3": np.zeros((ne, 2, nlev + 1)), "zxu": np.zeros((ne, nlev))}
    else:
        metrics = _terrain_metrics(mesh, zw, zgrid, mesh["deriv_two"])
    init = {
        "u": u, "w": w, "theta": theta, "rho": rho,
        "rho_base": rho_b, "theta_base": theta_b,
        "zz": metrics["zz"], "zgrid": zgrid,
        "zb": metrics["zb"], "zb3": metrics["zb3"],
        "zxu": metrics["zxu"],
        "scalars": scalars, "num_scalars": scalars.shape[-1], "qv": qv,
        "moist_start": 1, "moist_end": 1 if spec.qv_surface > 0.0 else 0,
        "u_init": np.full(nlev, float(spec.uv_init[0])), "v_init": np.full(nlev, float(spec.uv_init[1])),
        "t_init": theta_b.copy(), "qv_init": np.zeros(nlev),
        "dss": damping_coefficients(zgrid),
    }
    for k, v in vm.items():
        if k in ("dzw", "dzu"):
            init[k] = v
        else:
            init[k] = v
    return init


def make_case(spec: CaseSpec, radius: float = EARTH_RADIUS):
    """``(raw_init, raw_mesh)`` for ``spec``; the mesh carries the 2-D metric arrays too."""
    mesh = build_mesh(spec.level, radius)
    init = initial_state(mesh, spec, radius)
    # deriv_two / defc_* are init-file fields in MPAS; move them there
    for k in ("deriv_two", "defc_a", "defc_b"):
        init[k] = mesh.pop(k)
    return init, mesh


def write_case_files(spec: CaseSpec, directory, radius: float = EARTH_RADIUS, clobber: bool = False):
    """Write the synthetic case as an MPAS grid file and an initial-condition file
    (NetCDF-3, MPAS dimension and field names; ``netcdf_io.write_mpas_fields``), the pair
    ``load_initial_state(init_path, grid_path)`` reads.  Returns ``(init_path, grid_path)``."""
    import pathlib

    from .netcdf_io import write_mpas_fields
    d = pathlib.Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    init, grid = make_case(spec, radius)
    # an init_atmosphere output file carries the grid's fields too (readers take the mesh
    # dimensions from them)
    init = dict(grid, **init)
    init["nVertLevels"] = int(spec.nlev)
    tag = f"x1.{grid['nCells']}"
    grid_path, init_path = d / f"{tag}.grid.nc", d / f"{tag}.init.nc"
    write_mpas_fields(grid_path, grid, attrs={"sphere_radius": float(radius)}, clobber=clobber)
    write_mpas_fields(init_path, init, attrs={"sphere_radius": float(radius)}, clobber=clobber)
    return init_path, grid_path
