"""In-memory case loader: raw MPAS grid/init arrays -> the reference's runtime dictionaries.

Restates the derived-field synthesis of the reference loader
(``mpas_pytorch/ic_loader.py:1243 load_initial_state``) for arrays already in memory:
padding rows (:1079), inverse metrics and ``kiteForCell`` (:280), edge signs
(initialization.py:79), stencil trimming (:567-678), mesh scaling (initialization.py:203),
Pattern-C advection stencils from ``deriv_two`` (:358), ``zb_cell/zb3_cell`` (:214),
Rayleigh ``dss`` (:750, initialization.py:333) and RBF reconstruction coefficients
(:830, mesh_geometry.py:216).  Integer fields match the reference exactly; float fields
match to rounding (the RBF systems use LAPACK instead of MPAS's own elimination).
"""

from __future__ import annotations

import math
from typing import Any, Mapping

import numpy as np
import torch

from .cases import CaseSpec, make_case


def _pad(a: np.ndarray) -> np.ndarray:
    return np.concatenate([a, np.zeros((1,) + a.shape[1:], dtype=a.dtype)])


def _unit(v):
    n = np.sqrt(v[..., 0:1] ** 2 + v[..., 1:2] ** 2 + v[..., 2:3] ** 2)
    return v / n


def _dot(a, b):
    return a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1] + a[..., 2] * b[..., 2]


def _cross(a, b):
    return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1],
                     a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                     a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], -1)


def advective_stencils(coe, coc, neoc, deriv_two, dc, dv, nc, coef3):
    """advCellsForEdge / adv_coefs / adv_coefs_3rd from deriv_two (ic_loader.py:358-452)."""
    ne = coe.shape[0]
    maxe = coc.shape[1]
    c1, c2 = coe[:, 0], coe[:, 1]  # 1-based
    lists = np.zeros((ne, 2 + 2 * maxe), np.int64)
    lists[:, 0] = c1
    lists[:, 1] = c2
    count = np.full(ne, 2, np.int64)
    rows = np.arange(ne)

    def add_unique(cand, valid):
        present = np.any(lists == cand[:, None], axis=1)
        ok = valid & ~present
        lists[rows[ok], count[ok]] = cand[ok]
        count[ok] += 1

    n1 = neoc[c1 - 1]
    n2 = neoc[c2 - 1]
    for i in range(maxe):
        nb = coc[c1 - 1, i]
        add_unique(nb, (i < n1) & (nb != c2))
    for i in range(maxe):
        nb = coc[c2 - 1, i]
        add_unique(nb, i < n2)
    nmax = int(count.max())
    adv = np.zeros((ne, deriv_two.shape[-1]))
    adv3 = np.zeros((ne, deriv_two.shape[-1]))

    def pos(cell):
        return np.argmax(lists == cell[:, None], axis=1)

    p = pos(c1)
    adv[rows, p] += deriv_two[:, 0, 0]
    adv3[rows, p] += deriv_two[:, 0, 0]
    for i in range(maxe):
        ok = i < n1
        nb = np.where(ok, coc[c1 - 1, i], 0)
        p = pos(nb)
        cf = deriv_two[:, 0, i + 1]
        adv[rows[ok], p[ok]] += cf[ok]
        adv3[rows[ok], p[ok]] += cf[ok]
    p = pos(c2)
    adv[rows, p] += deriv_two[:, 1, 0]
    adv3[rows, p] -= deriv_two[:, 1, 0]
    for i in range(maxe):
        ok = i < n2
        nb = np.where(ok, coc[c2 - 1, i], 0)
        p = pos(nb)
        cf = deriv_two[:, 1, i + 1]
        adv[rows[ok], p[ok]] += cf[ok]
        adv3[rows[ok], p[ok]] -= cf[ok]
    active = np.arange(adv.shape[1])[None, :] < count[:, None]
    dc2 = (dc * dc)[:, None]
    adv = np.where(active, -dc2 * adv / 12.0, adv)
    adv3 = np.where(active, -dc2 * adv3 / 12.0, adv3)
    adv[rows, 0] += 0.5
    adv[rows, 1] += 0.5
    adv = np.where(active, adv * dv[:, None], adv)
    adv3 = np.where(active, adv3 * dv[:, None], adv3)
    adv3 = adv3 * coef3
    lists = np.where(np.arange(lists.shape[1])[None, :] < count[:, None], lists, 0)
    return lists[:, :nmax], count, adv[:, :nmax], adv3[:, :nmax]


def coeffs_reconstruct(xc, xe, nvec, eoc, neoc):
    """RBF reconstruction coefficients (mesh_geometry.py:216-343; MPAS mpas_init_reconstruct)."""
    nc, maxe = eoc.shape
    rhat = _unit(xc)
    first = eoc[:, 0] - 1
    en = nvec[first]
    x_hat = _unit(en - _dot(en, rhat)[:, None] * rhat)
    y_hat = _unit(_cross(rhat, x_hat))
    plane = np.stack([x_hat, y_hat], 1)
    coeffs = np.zeros((nc, maxe, 3))
    for npts in np.unique(neoc):
        ids = np.nonzero(neoc == npts)[0]
        e = eoc[ids, :npts] - 1
        cen = xc[ids]
        loc = xe[e]
        nrm = nvec[e]
        disp = cen[:, None, :] - loc
        radii = np.sqrt(disp[..., 0] ** 2 + disp[..., 1] ** 2 + disp[..., 2] ** 2)
        alpha = radii.sum(1) / npts
        pb = plane[ids]
        src = np.stack([_dot(loc, pb[:, a, None, :]) for a in range(2)], -1)
        uni = np.stack([_dot(nrm, pb[:, a, None, :]) for a in range(2)], -1)
        dst = np.stack([_dot(cen, pb[:, a, :]) for a in range(2)], -1)
        n = npts + 2
        mat = np.zeros((ids.size, n, n))
        rhs = np.zeros((ids.size, n, 2))
        d = src[:, :, None, :] - src[:, None, :, :]
        r2 = (d[..., 0] ** 2 + d[..., 1] ** 2) / (alpha ** 2)[:, None, None]
        rbf = 1.0 / np.sqrt(1.0 + r2)
        mat[:, :npts, :npts] = rbf * (uni[:, :, None, 0] * uni[:, None, :, 0] + uni[:, :, None, 1] * uni[:, None, :, 1])
        mat[:, :npts, npts:] = uni
        mat[:, npts:, :npts] = np.transpose(uni, (0, 2, 1))
        dd = dst[:, None, :] - src
        drbf = 1.0 / np.sqrt(1.0 + (dd[..., 0] ** 2 + dd[..., 1] ** 2) / (alpha ** 2)[:, None])
        rhs[:, :npts, :] = drbf[..., None] * uni
        rhs[:, npts, 0] = 1.0
        rhs[:, npts + 1, 1] = 1.0
        sol = np.linalg.solve(mat, rhs)
        coeffs[ids, :npts, :] = (pb[:, 0, None, :] * sol[:, :npts, 0, None]
                                 + pb[:, 1, None, :] * sol[:, :npts, 1, None])
    return coeffs


def load_arrays(init: Mapping[str, Any], grid: Mapping[str, Any], config: Mapping[str, Any] | None = None,
                as_torch: bool = True) -> dict:
    """Runtime state dictionary (mesh + state in one, like the reference's merged state)."""
    cfg = dict(config or {})
    nc, ne, nv = int(grid["nCells"]), int(grid["nEdges"]), int(grid["nVertices"])
    out: dict[str, Any] = {}
    for src in (grid, init):
        for k, v in src.items():
            if isinstance(v, np.ndarray) and v.ndim >= 1 and v.shape[0] in (nc, ne, nv):
                out[k] = _pad(v)
            else:
                out[k] = v
    nl = int(np.asarray(init["theta"]).shape[1])
    out["nVertLevels"] = nl
    maxe = int(grid["maxEdges"])
    # inverse metrics
    for s, t, n in (("areaCell", "invAreaCell", nc), ("areaTriangle", "invAreaTriangle", nv),
                    ("dvEdge", "invDvEdge", ne), ("dcEdge", "invDcEdge", ne)):
        src = out[s][:n]
        inv = np.zeros(n + 1)
        inv[:n] = np.where(src != 0, 1.0 / np.where(src != 0, src, 1.0), 0.0)
        out[t] = inv
    neoc = out["nEdgesOnCell"][:nc].astype(np.int64)
    voc = out["verticesOnCell"][:nc].astype(np.int64)
    cov = out["cellsOnVertex"][:nv].astype(np.int64)
    slot_ok = np.arange(maxe)[None, :] < neoc[:, None]
    cells = np.arange(1, nc + 1)
    gathered = cov[np.where(slot_ok, voc - 1, 0)]
    match = gathered == cells[:, None, None]
    kite = np.zeros((nc + 1, maxe), np.int32)
    kite[:nc] = np.where(slot_ok, np.argmax(match, axis=2) + 1, 0)
    out["kiteForCell"] = kite
    # edge signs
    eoc = out["edgesOnCell"][:nc].astype(np.int64)
    coe = out["cellsOnEdge"].astype(np.int64)
    sgn = np.zeros((nc + 1, maxe))
    e0 = np.where(slot_ok, eoc - 1, 0)
    sgn[:nc] = np.where(slot_ok, np.where(coe[e0, 0] == cells[:, None], 1.0, -1.0), 0.0)
    out["edgesOnCell_sign"] = sgn
    eov = out["edgesOnVertex"][:nv].astype(np.int64)
    voe = out["verticesOnEdge"].astype(np.int64)
    vs = np.zeros((nv + 1, eov.shape[1]))
    vs[:nv] = np.where(voe[eov - 1, 1] == np.arange(1, nv + 1)[:, None], 1.0, -1.0)
    out["edgesOnVertex_sign"] = vs
    # mesh scaling (meshDensity, config_h_ScaleWithMesh default)
    dens = out["meshDensity"]
    c1, c2 = coe[:ne, 0] - 1, coe[:ne, 1] - 1
    de = 0.5 * (dens[c1] + dens[c2])
    ms2 = np.ones(ne + 1)
    ms4 = np.ones(ne + 1)
    ms2[:ne] = np.where(de > 0, 1.0 / de ** 0.25, 1.0)
    ms4[:ne] = np.where(de > 0, 1.0 / de ** 0.75, 1.0)
    out["meshScalingDel2"], out["meshScalingDel4"] = ms2, ms4
    out["meshScalingRegionalCell"] = np.ones(nc + 1)
    out["meshScalingRegionalEdge"] = np.ones(ne + 1)
    out["bdyMaskCell"] = np.zeros(nc + 1, np.int32)
    out["bdyMaskEdge"] = np.zeros(ne + 1, np.int32)
    coef3 = float(cfg.get("config_coef_3rd_order", 0.25))
    out["coef_3rd_order"] = coef3
    out["c_s"] = float(cfg.get("config_smagorinsky_coef", 0.125))
    ns = int(np.asarray(init["scalars"]).shape[-1])
    out["num_scalars"] = ns
    out["moist_start"] = int(init.get("moist_start", 1))
    out["moist_end"] = int(init.get("moist_end", ns))
    # advection stencils
    lists, count, adv, adv3 = advective_stencils(coe[:ne], out["cellsOnCell"][:nc].astype(np.int64), neoc,
                                                 out["deriv_two"][:ne], out["dcEdge"][:ne],
                                                 out["dvEdge"][:ne], nc, coef3)
    w = adv.shape[1]
    out["advCellsForEdge"] = _pad(lists.astype(np.int32))
    out["nAdvCellsForEdge"] = _pad(count.astype(np.int32))
    out["adv_coefs"] = _pad(adv)
    out["adv_coefs_3rd"] = _pad(adv3)
    out["nAdvCellsMax"] = w
    # edgesOnEdge width
    m2 = int(out["nEdgesOnEdge"][:ne].max())
    out["edgesOnEdge"] = out["edgesOnEdge"][:, :m2]
    out["weightsOnEdge"] = out["weightsOnEdge"][:, :m2]
    out["maxEdges2"] = m2
    # zb_cell / zb3_cell from the edge-side metric
    side = (coe[e0, 1] == cells[:, None]).astype(np.int64)
    for name, scale in (("zb", 1.0), ("zb3", coef3)):
        src = out[name][:ne]
        g = src[e0, side]  # (nc, maxe, L+1)
        g = g * slot_ok[..., None]
        out[name + "_cell"] = _pad(g * scale)
    # Rayleigh damping coefficient: an initial-condition file's nonzero dss is kept as it
    # is (ic_loader.py:762-766), else computed (initialization.py:333)
    given = out.get("dss")
    keep = isinstance(given, np.ndarray) and given.shape == (nc + 1, nl) and bool(np.any(given[:nc] != 0))
    zgrid = out["zgrid"][:nc, : nl + 1]
    zt = zgrid[:, nl]
    zmid = 0.5 * (zgrid[:, :nl] + zgrid[:, 1:nl + 1])
    zd = float(cfg.get("config_zd", 22000.0))
    xnutr = float(cfg.get("config_xnutr", 0.2))
    arg = 0.5 * math.acos(-1.0) * (zmid - zd) / (zt[:, None] - zd)
    raw = xnutr * np.sin(arg) ** 2.0 / dens[:nc, None] ** 0.25
    if not keep:
        out["dss"] = _pad(np.where(zmid > zd, raw, 0.0))
    # reconstruction geometry
    xc = np.stack([out["xCell"][:nc], out["yCell"][:nc], out["zCell"][:nc]], -1)
    xe = np.stack([out["xEdge"][:ne], out["yEdge"][:ne], out["zEdge"][:ne]], -1)
    nvec = _unit(xc[c2] - xc[c1])
    out["edgeNormalVectors"] = _pad(nvec)
    out["localVerticalUnitVectors"] = _pad(_unit(xc))
    out["coeffs_reconstruct"] = _pad(coeffs_reconstruct(xc, xe, nvec, eoc, neoc))
    rhat = _unit(xc)
    en = nvec[eoc[:, 0] - 1]
    x_hat = _unit(en - _dot(en, rhat)[:, None] * rhat)
    out["cellTangentPlane"] = _pad(np.stack([x_hat, _unit(_cross(rhat, x_hat))], 1))
    out["rt_diabatic_tend"] = np.zeros((nc + 1, nl))
    out["nCells"], out["nEdges"], out["nVertices"] = nc, ne, nv
    if as_torch:
        out = {k: (torch.from_numpy(np.ascontiguousarray(v)) if isinstance(v, np.ndarray) else v)
               for k, v in out.items()}
    return out


def load_case(spec: CaseSpec, config: Mapping[str, Any] | None = None, as_torch: bool = True):
    """``(state, mesh)`` for a synthetic case; the state dictionary also carries the mesh."""
    init, grid = make_case(spec)
    st = load_arrays(init, grid, config, as_torch=as_torch)
    return st, st
