"""Per-stage numpy restatement of the reference's dynamics stages.

Every function takes one mapping ``a`` holding the reference stage's keyword
arguments (padded ``(N+1, ...)`` float64 arrays, 1-based connectivity, Python
scalars) and returns a dict with the reference's output keys.  Only active rows
(``[:N]``) of the outputs carry meaning; padding rows are left as the reference
leaves them where that is simple, otherwise zero.

Summation order follows the reference: per-entity slot loops in connectivity slot
order, accumulated left to right (``dynamics/stencil_ops.py:145-184``), with each
slot weight formed before it multiplies the gathered value.
"""

from __future__ import annotations

import math

import numpy as np

GRAVITY = 9.80616
RGAS = 287.0
RV = 461.6
CP = 1004.5
CV = 717.5
P0 = 100000.0
OMEGA = 7.29212e-5

def exner_pow(x, rcv):
    """x**rcv by the C library's scalar pow, element by element: what the reference's
    torch pow computes on its default (non-vectorised) CPU path, where NumPy's vectorised
    power may round the last bit differently."""
    x = np.asarray(x, dtype=np.float64)
    return np.fromiter((math.pow(v, rcv) for v in x.ravel()), np.float64, x.size).reshape(x.shape)


__all__ = [
    "idx0", "moist_coefficients", "vert_imp_coefs", "tridiagonal_solve",
    "acoustic_step", "divergence_damping", "smlstep_pert", "recover_large_step",
    "solve_diagnostics", "reconstruct_2d", "dyn_tend", "flux3", "flux4",
    "advance_scalars", "advance_scalars_mono",
]


def idx0(conn, n):
    """1-based connectivity -> 0-based rows; sentinels (0 or > n) -> padding row ``n``."""
    c = np.asarray(conn).astype(np.int64)
    return np.where((c >= 1) & (c <= n), c - 1, n)


def _i(a, k):
    v = a[k]
    return int(v.item()) if hasattr(v, "item") else int(v)


def _f(a, k):
    v = a[k]
    return float(v.item()) if hasattr(v, "item") else float(v)


def _sgn(x):
    """Fortran ``sign(1.0, x)``: +1 for x >= 0 (including +0), -1 for x < 0."""
    return np.where(x < 0.0, -1.0, 1.0)


# --------------------------------------------------------------------------------------
# moist coefficients  (dynamics/moist_coefficients.py:124)
# --------------------------------------------------------------------------------------

def moist_coefficients(a):
    """qtot = ordered sum of moist species; cqw = 1/(1+qtot_w); cqu = 1/(1+qtot_edge)."""
    nc, ne, nl = _i(a, "nCells"), _i(a, "nEdges"), _i(a, "nVertLevels")
    ms, me = _i(a, "moist_start"), _i(a, "moist_end")
    sc = a["scalars"]
    qtot = np.zeros((nc + 1, nl))
    for s in range(ms - 1, me):
        qtot[:nc] = qtot[:nc] + sc[:nc, :, s]
    cqw = np.zeros((nc + 1, nl + 1))
    cqw[:nc, 1:nl] = 1.0
    cqu = np.ones((ne + 1, nl))
    if me >= ms:
        cqw[:nc, 1:nl] = 1.0 / (1.0 + 0.5 * (qtot[:nc, 1:] + qtot[:nc, :-1]))
        coe = idx0(a["cellsOnEdge"][:ne], nc)
        q1 = qtot[coe[:, 0]]
        q2 = qtot[coe[:, 1]]
        cqu[:ne] = 1.0 / (1.0 + 0.5 * (q1 + q2))
    return {"qtot": qtot, "cqw": cqw, "cqu": cqu}


# --------------------------------------------------------------------------------------
# vertical implicit coefficients  (dynamics/vert_imp_coefs.py:188, factor :100)
# --------------------------------------------------------------------------------------

def vert_imp_coefs(a):
    """Column coefficients of the acoustic implicit solve and their Thomas factors.

    Returns the active-row (``(C, L)``; ``coftz (C, L+1)``) arrays the reference
    hands to the acoustic step under ``_vertical_implicit_coefficients_*_active``.
    """
    nc, nl = _i(a, "nCells"), _i(a, "nVertLevels")
    dts, epssm = _f(a, "dts"), _f(a, "epssm")
    g, rgas, cp = _f(a, "gravity"), _f(a, "rgas"), _f(a, "cp")
    dtseps = 0.5 * dts * (1.0 + epssm)
    rcv = rgas / (cp - rgas)
    c2 = cp * rcv
    rdzw = a["rdzw"][:nl]
    fzm = a["fzm"][:nl]
    fzp = a["fzp"][:nl]
    rdzu = a["rdzu"][:nl]
    zz = a["zz"][:nc, :nl]
    cqw = a["cqw"][:nc, :nl]
    p = a["p"][:nc, :nl]
    t = a["t"][:nc, :nl]
    rb = a["rb"][:nc, :nl]
    rtb = a["rtb"][:nc, :nl]
    pb = a["pb"][:nc, :nl]
    rt = a["rt"][:nc, :nl]
    qtot = a["qtot"][:nc, :nl]
    cofrz = dtseps * rdzw
    cofwr = np.zeros((nc, nl))
    cofwz = np.zeros((nc, nl))
    coftz = np.zeros((nc, nl + 1))
    cofwr[:, 1:] = 0.5 * dtseps * g * (fzm[1:] * zz[:, 1:] + fzp[1:] * zz[:, :-1])
    z_i = fzm[1:] * zz[:, 1:] + fzp[1:] * zz[:, :-1]
    p_i = fzm[1:] * p[:, 1:] + fzp[1:] * p[:, :-1]
    t_i = fzm[1:] * t[:, 1:] + fzp[1:] * t[:, :-1]
    cofwz[:, 1:] = dtseps * c2 * z_i * rdzu[1:nl] * cqw[:, 1:] * p_i
    coftz[:, 1:nl] = dtseps * t_i
    cofwt = 0.5 * dtseps * rcv * zz * g * rb / (1.0 + qtot) * p / ((rtb + rt) * pb)
    a_tri = np.zeros((nc, nl))
    b_tri = np.ones((nc, nl))
    c_tri = np.zeros((nc, nl))
    a_tri[:, 1:] = (-cofwz[:, 1:] * coftz[:, :nl - 1] * rdzw[:nl - 1] * zz[:, :nl - 1]
                    + cofwr[:, 1:] * cofrz[:nl - 1]
                    - cofwt[:, :nl - 1] * coftz[:, :nl - 1] * rdzw[:nl - 1])
    b_tri[:, 1:] = (1.0 + cofwz[:, 1:] * (coftz[:, 1:nl] * rdzw[1:] * zz[:, 1:]
                                          + coftz[:, 1:nl] * rdzw[:nl - 1] * zz[:, :nl - 1])
                    - coftz[:, 1:nl] * (cofwt[:, 1:] * rdzw[1:] - cofwt[:, :nl - 1] * rdzw[:nl - 1])
                    + cofwr[:, 1:] * (cofrz[1:] - cofrz[:nl - 1]))
    c_tri[:, 1:] = (-cofwz[:, 1:] * coftz[:, 2:nl + 1] * rdzw[1:] * zz[:, 1:]
                    - cofwr[:, 1:] * cofrz[1:]
                    + cofwt[:, 1:] * coftz[:, 2:nl + 1] * rdzw[1:])
    alpha = np.zeros((nc, nl))
    gamma = np.zeros((nc, nl))
    for k in range(1, nl):
        alpha[:, k] = 1.0 / (b_tri[:, k] - a_tri[:, k] * gamma[:, k - 1])
        gamma[:, k] = c_tri[:, k] * alpha[:, k]
    pre = "_vertical_implicit_coefficients_"
    return {"cofrz": cofrz, pre + "cofwr_active": cofwr, pre + "cofwz_active": cofwz,
            pre + "coftz_active": coftz, pre + "cofwt_active": cofwt,
            pre + "a_tri_active": a_tri, pre + "alpha_tri_active": alpha,
            pre + "gamma_tri_active": gamma}


def tridiagonal_solve(a_tri, alpha, gamma, rhs):
    """Thomas sweeps on factored columns (autodiff/tridiagonal_solve.py:56-63).

    ``rhs`` is ``(C, L+1)``; levels 1..L-1 (0-based) are solved; level 0 and L are
    boundary values (forward sweep starts at k=1, back substitution runs k=L-1..0).
    """
    x = rhs.copy()
    nl = a_tri.shape[1]
    for k in range(1, nl):
        x[:, k] = (x[:, k] - a_tri[:, k] * x[:, k - 1]) * alpha[:, k]
    for k in range(nl - 1, -1, -1):
        x[:, k] = x[:, k] - gamma[:, k] * x[:, k + 1]
    return x


# --------------------------------------------------------------------------------------
# acoustic substep  (dynamics/acoustic_step.py:1297; edge update :576; cell fluxes :456;
#                    RHS :675; solve + Rayleigh + post-solve :772)
# --------------------------------------------------------------------------------------

def acoustic_step(a):
    nc, ne, nl = _i(a, "nCells"), _i(a, "nEdges"), _i(a, "nVertLevels")
    small_step = _i(a, "small_step")
    dts, epssm, resm, c2 = _f(a, "dts"), _f(a, "epssm"), _f(a, "resm"), _f(a, "c2")
    pre = "_vertical_implicit_coefficients_"
    coe = idx0(a["cellsOnEdge"][:ne], nc)
    c1, c2i = coe[:, 0], coe[:, 1]
    ru_p = a["ru_p"].copy()
    ru_avg = a["ruAvg"].copy()
    rtheta_pp = a["rtheta_pp"]
    rho_pp = a["rho_pp"]
    if small_step != 1:
        zz, exner = a["zz"], a["exner"]
        pgrad = ((rtheta_pp[c2i] - rtheta_pp[c1]) * a["invDcEdge"][:ne, None]) / (0.5 * (zz[c2i] + zz[c1]))
        pgrad = a["cqu"][:ne] * 0.5 * c2 * (exner[c1] + exner[c2i]) * pgrad
        pgrad = pgrad + 0.5 * a["zxu"][:ne] * GRAVITY * (rho_pp[c1] + rho_pp[c2i])
        ru_p[:ne] = ru_p[:ne] + dts * (a["tend_ru"][:ne] - (1.0 - a["specZoneMaskEdge"][:ne, None]) * pgrad)
        ru_avg[:ne] = ru_avg[:ne] + ru_p[:ne]
    else:
        ru_p[:ne] = dts * a["tend_ru"][:ne]
        ru_avg[:ne] = ru_p[:ne]

    # the saved pre-update value is taken after the small_step == 1 reset
    rtheta_pp_old = a["rtheta_pp_old"].copy()
    rtheta_pp_old[:nc] = 0.0 if small_step == 1 else rtheta_pp[:nc]

    rho_pp_in = rho_pp[:nc].copy()
    rtheta_pp_in = rtheta_pp[:nc].copy()
    rw_p = a["rw_p"].copy()
    ww = a["wwAvg"].copy()
    if small_step == 1:
        rho_pp_in[:] = 0.0
        rtheta_pp_in[:] = 0.0
        rw_p[:nc] = 0.0
        ww[:nc] = 0.0

    # cell flux sums in edgesOnCell slot order
    theta_m = a["theta_m"]
    eoc = idx0(a["edgesOnCell"][:nc], ne)
    n_eoc = np.asarray(a["nEdgesOnCell"][:nc]).astype(np.int64)
    sign = a["edgesOnCell_sign"][:nc]
    inv_area = a["invAreaCell"][:nc]
    dv = a["dvEdge"]
    rs = None
    ts = None
    for j in range(eoc.shape[1]):
        valid = (j < n_eoc) & (eoc[:, j] < ne)
        e = np.where(valid, eoc[:, j], 0)
        w = np.where(valid, sign[:, j] * dv[e], 0.0)
        flux = dts * w[:, None] * ru_p[e] * inv_area[:, None]
        th_e = 0.5 * (theta_m[c2i[e]] + theta_m[c1[e]])
        flux = flux * valid[:, None]
        th_e = th_e * valid[:, None]
        rs = -flux if rs is None else rs + (-flux)
        ts = -(flux * th_e) if ts is None else ts + (-(flux * th_e))

    cofrz = a["cofrz"][:nl]
    rdzw = a["rdzw"][:nl]
    coftz = a[pre + "coftz_active"]
    cofwz = a[pre + "cofwz_active"]
    cofwr = a[pre + "cofwr_active"]
    cofwt = a[pre + "cofwt_active"]
    zz = a["zz"][:nc, :nl]
    rwp = rw_p[:nc]
    rs = rho_pp_in + dts * a["tend_rho"][:nc] + rs - cofrz[None, :] * resm * (rwp[:, 1:] - rwp[:, :nl])
    ts = (rtheta_pp_in + dts * a["tend_rt"][:nc] + ts
          - resm * rdzw[None, :] * (coftz[:, 1:] * rwp[:, 1:] - coftz[:, :nl] * rwp[:, :nl]))
    wwc = ww[:nc].copy()
    wwc[:, 1:nl] = wwc[:, 1:nl] + 0.5 * (1.0 - epssm) * rwp[:, 1:nl]
    rhs = rwp.copy()
    rhs[:, 1:nl] = (rwp[:, 1:nl] + dts * a["tend_rw"][:nc, 1:nl]
                    - cofwz[:, 1:] * ((zz[:, 1:] * ts[:, 1:] - zz[:, :-1] * ts[:, :-1])
                                      + resm * (zz[:, 1:] * rtheta_pp_in[:, 1:] - zz[:, :-1] * rtheta_pp_in[:, :-1]))
                    - cofwr[:, 1:] * ((rs[:, 1:] + rs[:, :-1]) + resm * (rho_pp_in[:, 1:] + rho_pp_in[:, :-1]))
                    + cofwt[:, 1:] * (ts[:, 1:] + resm * rtheta_pp_in[:, 1:])
                    + cofwt[:, :-1] * (ts[:, :-1] + resm * rtheta_pp_in[:, :-1]))
    sol = tridiagonal_solve(a[pre + "a_tri_active"], a[pre + "alpha_tri_active"],
                            a[pre + "gamma_tri_active"], rhs)
    fzm, fzp = a["fzm"][:nl], a["fzp"][:nl]
    zz_i = fzm[1:] * zz[:, 1:] + fzp[1:] * zz[:, :-1]
    rho_zz = a["rho_zz"][:nc, :nl]
    rho_i = fzm[1:] * rho_zz[:, 1:] + fzp[1:] * rho_zz[:, :-1]
    dss = a["dss"][:nc, :nl]
    rw_delta = a["rw_save"][:nc, 1:nl] - a["rw"][:nc, 1:nl]
    sol[:, 1:nl] = (sol[:, 1:nl] + rw_delta - dts * dss[:, 1:] * zz_i * rho_i * a["w"][:nc, 1:nl]) \
        / (1.0 + dts * dss[:, 1:]) - rw_delta
    wwc[:, 1:nl] = wwc[:, 1:nl] + 0.5 * (1.0 + epssm) * sol[:, 1:nl]
    rho_new = rs - cofrz[None, :] * (sol[:, 1:] - sol[:, :nl])
    rt_new = ts - rdzw[None, :] * (coftz[:, 1:] * sol[:, 1:] - coftz[:, :nl] * sol[:, :nl])
    rw_p[:nc] = sol
    ww[:nc] = wwc
    rho_pp_out = a["rho_pp"].copy()
    rho_pp_out[:nc] = rho_new
    rtheta_pp_out = a["rtheta_pp"].copy()
    rtheta_pp_out[:nc] = rt_new
    return {"ru_p": ru_p, "ruAvg": ru_avg, "rho_pp": rho_pp_out, "rtheta_pp": rtheta_pp_out,
            "rtheta_pp_old": rtheta_pp_old, "rw_p": rw_p, "wwAvg": ww,
            "w": a["w"], "exner": a["exner"]}


# --------------------------------------------------------------------------------------
# divergence damping  (dynamics/divergence_damping.py:299, region :187)
# --------------------------------------------------------------------------------------

def divergence_damping(a):
    nc, ne = _i(a, "nCells"), _i(a, "nEdges")
    dts = _f(a, "dts")
    coef = 2.0 * _f(a, "config_smdiv") * _f(a, "config_len_disp") / dts
    coe = idx0(a["cellsOnEdge"][:ne], nc)
    c1, c2 = coe[:, 0], coe[:, 1]
    rt, rto, th = a["rtheta_pp"], a["rtheta_pp_old"], a["theta_m"]
    d1 = -(rt[c1] - rto[c1])
    d2 = -(rt[c2] - rto[c2])
    ru_p = a["ru_p"].copy()
    ru_p[:ne] = ru_p[:ne] + coef * (d2 - d1) * (1.0 - a["specZoneMaskEdge"][:ne, None]) / (th[c1] + th[c2])
    return {"ru_p": ru_p}


# --------------------------------------------------------------------------------------
# small-step perturbation: w tendency -> omega tendency  (dynamics/smlstep_pert.py:373)
# --------------------------------------------------------------------------------------

def smlstep_pert(a):
    nc, ne, nl = _i(a, "nCells"), _i(a, "nEdges"), _i(a, "nVertLevels")
    fzm, fzp = a["fzm"][:nl], a["fzp"][:nl]
    wt = a["w_tend"].copy()
    ut = a["u_tend"]
    eoc = idx0(a["edgesOnCell"][:nc], ne)
    n_eoc = np.asarray(a["nEdgesOnCell"][:nc]).astype(np.int64)
    sign = a["edgesOnCell_sign"][:nc]
    zb = a["zb_cell"]
    zb3 = a["zb3_cell"]
    acc = wt[:nc, 1:nl].copy()
    for j in range(eoc.shape[1]):
        valid = (j < n_eoc) & (eoc[:, j] < ne)
        e = np.where(valid, eoc[:, j], 0)
        u_i = fzm[1:] * ut[e, 1:nl] + fzp[1:] * ut[e, :nl - 1]
        flux = sign[:, j, None] * u_i
        coef = zb[:nc, j, 1:nl] + _sgn(ut[e, 1:nl]) * zb3[:nc, j, 1:nl]
        acc = acc - np.where(valid[:, None], coef * flux, 0.0)
    zz = a["zz"][:nc, :nl]
    wt[:nc, 1:nl] = (fzm[1:] * zz[:, 1:] + fzp[1:] * zz[:, :-1]) * acc
    return {"w_tend": wt}


# --------------------------------------------------------------------------------------
# large-step recovery  (dynamics/recover_large_step.py:1090, numeric :516, slots :329)
# --------------------------------------------------------------------------------------

def recover_large_step(a):
    nc, ne, nl = _i(a, "nCells"), _i(a, "nEdges"), _i(a, "nVertLevels")
    rk_step, ns = _i(a, "rk_step"), _i(a, "ns")
    dt = _f(a, "dt")
    cf1, cf2, cf3 = _f(a, "cf1"), _f(a, "cf2"), _f(a, "cf3")
    inv_ns = 1.0 / float(ns)
    fzm, fzp = a["fzm"][:nl], a["fzp"][:nl]
    S = lambda k: a[k][:nc, :nl]
    rho_p = S("rho_p_save") + S("rho_pp")
    rho_zz = rho_p + S("rho_base")
    if rk_step == 3:
        rtheta_p = S("rtheta_p_save") + S("rtheta_pp") - dt * rho_zz * S("rt_diabatic_tend")
    else:
        rtheta_p = S("rtheta_p_save") + S("rtheta_pp")
    theta_m = (rtheta_p + S("rtheta_base")) / rho_zz
    out = {}
    if rk_step == 3:
        rcv = RGAS / (CP - RGAS)
        zz = S("zz")
        exner = exner_pow(zz * (RGAS / P0) * (rtheta_p + S("rtheta_base")), rcv)
        pressure_p = zz * RGAS * (exner * rtheta_p + S("rtheta_base") * (exner - S("exner_base")))
        out["exner"] = np.concatenate([exner, np.zeros((1, nl))])
        out["pressure_p"] = np.concatenate([pressure_p, np.zeros((1, nl))])
    coe = idx0(a["cellsOnEdge"][:ne], nc)
    rz_pad = np.concatenate([rho_zz, np.ones((1, nl))])
    ru_save = a["ru_save"][:ne]
    ru_avg = ru_save + a["ruAvg"][:ne] * inv_ns
    ru = ru_save + a["ru_p"][:ne]
    u = 2.0 * ru / (rz_pad[coe[:, 0]] + rz_pad[coe[:, 1]])
    zz = a["zz"][:nc, :nl]
    ww_mid = a["rw_save"][:nc, 1:nl] + a["wwAvg"][:nc, 1:nl] * inv_ns
    rw_mid = a["rw_save"][:nc, 1:nl] + a["rw_p"][:nc, 1:nl]
    w_mid = rw_mid / (fzm[1:] * zz[:, 1:] + fzp[1:] * zz[:, :-1])
    eoc = idx0(a["edgesOnCell"][:nc], ne)
    n_eoc = np.asarray(a["nEdgesOnCell"][:nc]).astype(np.int64)
    sign = a["edgesOnCell_sign"][:nc]
    zb = a["zb_cell"]
    zb3 = a["zb3_cell"]
    ru_pad = np.concatenate([ru, np.zeros((1, nl))])
    surf = None
    interior = w_mid
    for j in range(eoc.shape[1]):
        valid = (j < n_eoc) & (eoc[:, j] < ne)
        e = np.where(valid, eoc[:, j], ne)
        rs = ru_pad[e]
        fs = cf1 * rs[:, 0] + cf2 * rs[:, 1] + cf3 * rs[:, 2]
        cs = zb[:nc, j, 0] + _sgn(fs) * zb3[:nc, j, 0]
        sc = np.where(valid, sign[:, j] * cs * fs, 0.0)
        surf = sc if surf is None else surf + sc
        fi = fzm[1:] * rs[:, 1:nl] + fzp[1:] * rs[:, :nl - 1]
        ci = zb[:nc, j, 1:nl] + _sgn(fi) * zb3[:nc, j, 1:nl]
        interior = interior + np.where(valid[:, None], sign[:, j, None] * ci * fi, 0.0)
    w = np.zeros((nc + 1, nl + 1))
    w[:nc, 0] = surf / (cf1 * rho_zz[:, 0] + cf2 * rho_zz[:, 1] + cf3 * rho_zz[:, 2])
    w[:nc, 1:nl] = interior / (fzm[1:] * rho_zz[:, 1:] + fzp[1:] * rho_zz[:, :-1])

    def pad(x, rows):
        o = np.zeros((rows + 1,) + x.shape[1:])
        o[:rows] = x
        return o

    rw = a["rw_save"].copy()
    rw[:nc, 1:nl] = rw_mid
    ww = a["wwAvg"].copy()
    ww[:nc, 1:nl] = ww_mid
    out.update({"rho_p": pad(rho_p, nc), "rho_zz": pad(rho_zz, nc), "rtheta_p": pad(rtheta_p, nc),
                "theta_m": pad(theta_m, nc), "u": pad(u, ne), "ru": pad(ru, ne),
                "ruAvg": pad(ru_avg, ne), "w": w, "rw": rw, "wwAvg": ww})
    return out


# --------------------------------------------------------------------------------------
# diagnostics  (dynamics/solve_diagnostics.py:1052, composition :531, payload :280-460)
# --------------------------------------------------------------------------------------

def solve_diagnostics(a):
    nc, ne, nv, nl = _i(a, "nCells"), _i(a, "nEdges"), _i(a, "nVertices"), _i(a, "nVertLevels")
    rk_step = _i(a, "rk_step")
    dt, apvm = _f(a, "dt"), _f(a, "config_apvm_upwinding")
    u = a["u"]
    h = a["h"]
    coe = idx0(a["cellsOnEdge"][:ne], nc)
    voe = idx0(a["verticesOnEdge"][:ne], nv)
    dc, dv = a["dcEdge"], a["dvEdge"]
    h_edge = 0.5 * (h[coe[:, 0]] + h[coe[:, 1]])
    ke_edge = (dc[:ne] * dv[:ne])[:, None] * (u[:ne] ** 2)
    eov = idx0(a["edgesOnVertex"][:nv], ne)
    eov_sign = a["edgesOnVertex_sign"][:nv]
    vort = None
    kev = None
    for j in range(eov.shape[1]):
        valid = eov[:, j] < ne
        e = np.where(valid, eov[:, j], 0)
        wgt = np.where(valid, eov_sign[:, j] * dc[e], 0.0)
        c = wgt[:, None] * u[e]
        vort = c if vort is None else vort + c
        kc = np.where(valid[:, None], ke_edge[e], 0.0)
        kev = kc if kev is None else kev + kc
    vort = vort * a["invAreaTriangle"][:nv, None]
    ke_vertex = 0.25 * a["invAreaTriangle"][:nv, None] * kev
    eoc = idx0(a["edgesOnCell"][:nc], ne)
    n_eoc = np.asarray(a["nEdgesOnCell"][:nc]).astype(np.int64)
    sign = a["edgesOnCell_sign"][:nc]
    div = None
    ke = None
    for j in range(eoc.shape[1]):
        valid = (j < n_eoc) & (eoc[:, j] < ne)
        e = np.where(valid, eoc[:, j], 0)
        wgt = np.where(valid, sign[:, j] * dv[e], 0.0)
        c = wgt[:, None] * u[e]
        div = c if div is None else div + c
        kw = np.where(valid, 0.25, 0.0)
        kc = kw[:, None] * ke_edge[e]
        ke = kc if ke is None else ke + kc
    inv_area = a["invAreaCell"][:nc, None]
    div = div * inv_area
    ke = ke * inv_area
    ke_fact = 1.0 - 0.375
    ke = ke_fact * ke
    voc = idx0(a["verticesOnCell"][:nc], nv)
    kite = np.asarray(a["kiteForCell"][:nc]).astype(np.int64)
    kites = a["kiteAreasOnVertex"]
    nkite = kites.shape[1]
    cell_vert_valid = []
    cell_vert_w = []
    for j in range(voc.shape[1]):
        valid = (j < n_eoc) & (voc[:, j] < nv) & (kite[:, j] >= 1) & (kite[:, j] <= nkite)
        vv = np.where(valid, voc[:, j], 0)
        kk = np.where(valid, kite[:, j] - 1, 0)
        wgt = np.where(valid, kites[vv, kk], 0.0)
        cell_vert_valid.append((valid, vv))
        cell_vert_w.append(wgt)
        c = (1.0 - ke_fact) * wgt[:, None]
        c = c * ke_vertex[vv]
        c = c * inv_area
        ke = ke + np.where(valid[:, None], c, 0.0)
    pv_vertex = a["fVertex"][:nv, None] + vort
    pv_edge = 0.5 * (pv_vertex[voe[:, 0]] + pv_vertex[voe[:, 1]]) if nv > 0 else None
    if rk_step == 3:
        eoe = idx0(a["edgesOnEdge"][:ne], ne)
        n_eoe = np.asarray(a["nEdgesOnEdge"][:ne]).astype(np.int64)
        woe = a["weightsOnEdge"][:ne]
        v = None
        for j in range(eoe.shape[1]):
            valid = (j < n_eoe) & (eoe[:, j] < ne)
            e = np.where(valid, eoe[:, j], 0)
            wgt = np.where(valid, woe[:, j], 0.0)
            c = wgt[:, None] * u[e]
            v = c if v is None else v + c
    else:
        v = a["v_in"][:ne]
    if apvm > 0.0:
        pvc = None
        for j, (valid, vv) in enumerate(cell_vert_valid):
            c = cell_vert_w[j][:, None] * pv_vertex[vv]
            c = c * inv_area
            c = np.where(valid[:, None], c, 0.0)
            pvc = c if pvc is None else pvc + c
        pvc_pad = np.concatenate([pvc, np.zeros((1, nl))])
        pvv_pad = np.concatenate([pv_vertex, np.zeros((1, nl))])
        grad_pvt = (pvv_pad[voe[:, 1]] - pvv_pad[voe[:, 0]]) * a["invDvEdge"][:ne, None]
        grad_pvn = (pvc_pad[coe[:, 1]] - pvc_pad[coe[:, 0]]) * a["invDcEdge"][:ne, None]
        delta = (apvm * dt) * (v * grad_pvt + u[:ne] * grad_pvn)
        pv_edge = pv_edge - delta

    def pad(x, rows):
        o = np.zeros((rows + 1,) + x.shape[1:])
        o[:rows] = x
        return o

    return {"h_edge": pad(h_edge, ne), "v": pad(v, ne), "divergence": pad(div, nc),
            "vorticity": pad(vort, nv), "ke": pad(ke, nc), "pv_edge": pad(pv_edge, ne)}


# --------------------------------------------------------------------------------------
# cell-centre wind reconstruction  (dynamics/vector_reconstruction.py:311)
# --------------------------------------------------------------------------------------

def reconstruct_2d(a):
    nc, ne, nl = _i(a, "nCells"), _i(a, "nEdges"), _i(a, "nVertLevels")
    u = a["u"]
    coeffs = a["coeffs_reconstruct"][:nc]
    eoc = idx0(a["edgesOnCell"][:nc], ne)
    n_eoc = np.asarray(a["nEdgesOnCell"][:nc]).astype(np.int64)
    acc = np.zeros((nc, nl, 3))
    first = True
    for j in range(eoc.shape[1]):
        valid = (j < n_eoc) & (eoc[:, j] < ne)
        e = np.where(valid, eoc[:, j], 0)
        c = coeffs[:, j, None, :] * u[e][:, :, None]
        c = np.where(valid[:, None, None], c, 0.0)
        acc = c if first else acc + c
        first = False
    x, y, z = acc[..., 0], acc[..., 1], acc[..., 2]
    lat = a["latCell"][:nc, None]
    lon = a["lonCell"][:nc, None]
    clat, slat, clon, slon = np.cos(lat), np.sin(lat), np.cos(lon), np.sin(lon)
    zonal = -x * slon + y * clon
    merid = -(x * clon + y * slon) * slat + z * clat

    def pad(v):
        o = np.zeros((nc + 1, nl))
        o[:nc] = v
        return o

    return {"uReconstructX": pad(x), "uReconstructY": pad(y), "uReconstructZ": pad(z),
            "uReconstructZonal": pad(zonal), "uReconstructMeridional": pad(merid),
            "ur_cell": pad(zonal), "vr_cell": pad(merid)}


# --------------------------------------------------------------------------------------
# large-step tendencies  (dynamics/dyn_tend.py:10836, composition :9390; sections at
# :9925 kdiff, :9963 tend_rho, :9993 tend_u, :10075 u mixing, :10316 w advection,
# :10355 w mixing, :10386 w vertical, :10442 theta advection, :10544 theta mixing,
# :10679 theta vertical; flux3/flux4 :839/:853)
# --------------------------------------------------------------------------------------

def flux4(qm2, qm1, q0, qp1, ua):
    return ua * (7.0 * (q0 + qm1) - (qp1 + qm2)) / 12.0


def flux3(qm2, qm1, q0, qp1, ua, coef3):
    return flux4(qm2, qm1, q0, qp1, ua) + coef3 * np.abs(ua) * ((qp1 - qm2) - 3.0 * (q0 - qm1)) / 12.0


def dyn_tend(a):
    nc, ne, nv, nl = _i(a, "nCells"), _i(a, "nEdges"), _i(a, "nVertices"), _i(a, "nVertLevels")
    rk_step = _i(a, "rk_step")
    dt = _f(a, "dt")
    coef3 = _f(a, "coef_3rd_order")
    c_s = _f(a, "c_s")
    len_disp = _f(a, "config_len_disp")
    del4u_div = _f(a, "config_del4u_div_factor")
    inv_dt = 1.0 / dt
    prandtl_inv = 1.0
    mixing = str(a["config_horiz_mixing"])
    if mixing == "2d_smagorinsky":
        h_mom_eddy_visc4 = _f(a, "config_visc4_2dsmag") * len_disp ** 3
        h_theta_eddy_visc4 = h_mom_eddy_visc4
    else:
        h_mom_eddy_visc4 = _f(a, "config_h_mom_eddy_visc4")
        h_theta_eddy_visc4 = _f(a, "config_h_theta_eddy_visc4")

    coe = idx0(a["cellsOnEdge"][:ne], nc)
    e1, e2 = coe[:, 0], coe[:, 1]
    voe = idx0(a["verticesOnEdge"][:ne], nv)
    eoc = idx0(a["edgesOnCell"][:nc], ne)
    n_eoc = np.asarray(a["nEdgesOnCell"][:nc]).astype(np.int64)
    sign = a["edgesOnCell_sign"][:nc]
    dv, dc = a["dvEdge"], a["dcEdge"]
    inv_dc, inv_dv = a["invDcEdge"], a["invDvEdge"]
    inv_area = a["invAreaCell"]
    fzm, fzp = a["fzm"][:nl], a["fzp"][:nl]
    rdzw, rdzu = a["rdzw"][:nl], a["rdzu"][:nl]
    u, v, w = a["u"], a["v"], a["w"]
    ru, rw = a["ru"], a["rw"]
    rho_edge = a["rho_edge"]
    theta_m = a["theta_m"]
    kdiff_in = a.get("kdiff_in")

    def slots():
        for j in range(eoc.shape[1]):
            valid = (j < n_eoc) & (eoc[:, j] < ne)
            yield j, valid, np.where(valid, eoc[:, j], 0)

    zpad = lambda x: np.concatenate([x, np.zeros((1,) + x.shape[1:])])

    # ---- Smagorinsky eddy viscosity (rk_step 1) ----
    if rk_step == 1:
        kdiff = np.zeros((nc + 1, nl))
        if mixing == "2d_smagorinsky":
            d_diag = np.zeros((nc, nl))
            d_off = np.zeros((nc, nl))
            for j, valid, e in slots():
                ca = a["defc_a"][:nc, j][:, None]
                cb = a["defc_b"][:nc, j][:, None]
                dd = (d_diag + ca * u[e]) - cb * v[e]
                do = (d_off + cb * u[e]) + ca * v[e]
                d_diag = np.where(valid[:, None], dd, d_diag)
                d_off = np.where(valid[:, None], do, d_off)
            kdiff[:nc] = np.minimum((c_s * len_disp) ** 2 * np.sqrt(d_diag ** 2 + d_off ** 2),
                                    (0.01 * len_disp ** 2) * inv_dt)
        else:  # 2d_fixed: the theta coefficient everywhere (dyn_tend.py:3420-3427)
            kdiff[:nc] = _f(a, "config_h_theta_eddy_visc2")
        cam, ncam = _f(a, "config_mpas_cam_coef"), _i(a, "config_number_cam_damping_levels")
        if cam > 0.0 and ncam > 0:  # CAM-style top-level damping (dyn_tend.py:3434-3456)
            base = 4.0 * 2.0833 * len_disp * cam
            for k in range(nl - ncam, nl):
                kdiff[:nc, k] = np.maximum(kdiff[:nc, k], base * (1.0 - float(nl - (k + 1)) / float(ncam)))
    else:
        kdiff = kdiff_in

    # ---- density tendency ----
    h_div = None
    for j, valid, e in slots():
        wgt = np.where(valid, sign[:, j] * dv[e], 0.0)[:, None]
        c = wgt * ru[e]
        h_div = c if h_div is None else h_div + c
    h_div = h_div * inv_area[:nc, None]
    qtot = a["qtot"]
    if rk_step == 1:
        tend_rho = zpad(-h_div - rdzw[None, :] * (rw[:nc, 1:] - rw[:nc, :nl]))
    else:
        tend_rho = a["tend_rho_in"].copy()
    dpdz = np.zeros((nc + 1, nl))
    dpdz[:nc] = -GRAVITY * (a["rb"][:nc] * qtot[:nc] + a["rr_save"][:nc] * (1.0 + qtot[:nc]))
    h_div_p = zpad(h_div)

    # ---- u tendency ----
    zz = a["zz"]
    pp = a["pp"]
    if rk_step == 1:
        tend_u_euler = np.zeros((ne + 1, nl))
        tend_u_euler[:ne] = -a["cqu"][:ne] * ((pp[e2] - pp[e1]) * inv_dc[:ne, None] / (0.5 * (zz[e2] + zz[e1]))
                                             - 0.5 * a["zxu"][:ne] * (dpdz[e1] + dpdz[e2]))
    else:
        tend_u_euler = a["tend_u_euler_in"].copy()
    rw_e = 0.5 * (rw[e1] + rw[e2])
    wduz = np.zeros((ne, nl + 1))
    wduz[:, 1] = rw_e[:, 1] * (fzm[1] * u[:ne, 1] + fzp[1] * u[:ne, 0])
    for k in range(2, nl - 1):
        wduz[:, k] = flux3(u[:ne, k - 2], u[:ne, k - 1], u[:ne, k], u[:ne, k + 1], rw_e[:, k], 1.0)
    k = nl - 1
    wduz[:, k] = rw_e[:, k] * (fzm[k] * u[:ne, k] + fzp[k] * u[:ne, k - 1])
    tend_u = -rdzw[None, :] * (wduz[:, 1:] - wduz[:, :nl])
    eoe = idx0(a["edgesOnEdge"][:ne], ne)
    n_eoe = np.asarray(a["nEdgesOnEdge"][:ne]).astype(np.int64)
    woe = a["weightsOnEdge"][:ne]
    pv_edge = a["pv_edge"]
    q = None
    for j in range(eoe.shape[1]):
        valid = (j < n_eoe) & (eoe[:, j] < ne)
        e = np.where(valid, eoe[:, j], 0)
        workpv = 0.5 * (pv_edge[:ne] + pv_edge[e])
        c = np.where(valid, woe[:, j], 0.0)[:, None] * u[e] * workpv
        q = c if q is None else q + c
    ke = a["ke"]
    tend_u = tend_u + rho_edge[:ne] * (q - (ke[e2] - ke[e1]) * inv_dc[:ne, None]) \
        - u[:ne] * 0.5 * (h_div_p[e1] + h_div_p[e2])

    if rk_step == 1:
        div, vort = a["divergence"], a["vorticity"]
        v1, v2 = voe[:, 0], voe[:, 1]
        r_dc = inv_dc[:ne, None]
        r_dv = np.minimum(inv_dv[:ne], 4.0 * inv_dc[:ne])[:, None]
        u_diff = (div[e2] - div[e1]) * r_dc - (vort[v2] - vort[v1]) * r_dv
        delsq_u = u_diff
        kdiffu = 0.5 * (kdiff[e1] + kdiff[e2])
        tend_u_euler[:ne] = tend_u_euler[:ne] + rho_edge[:ne] * kdiffu * u_diff * a["meshScalingDel2"][:ne, None]
        if h_mom_eddy_visc4 > 0.0:
            eov = idx0(a["edgesOnVertex"][:nv], ne)
            eov_sign = a["edgesOnVertex_sign"][:nv]
            dsv = None
            for j in range(eov.shape[1]):
                valid = eov[:, j] < ne
                e = np.where(valid, eov[:, j], 0)
                es = np.where(valid, a["invAreaTriangle"][:nv] * dc[e] * eov_sign[:, j], 0.0)[:, None]
                c = es * delsq_u[e]
                dsv = c if dsv is None else dsv + c
            dsd = None
            for j, valid, e in slots():
                es = np.where(valid, inv_area[:nc] * dv[e] * sign[:, j], 0.0)[:, None]
                c = es * delsq_u[e]
                dsd = c if dsd is None else dsd + c
            dsv = zpad(dsv)
            dsd = zpad(dsd)
            u_mix = a["meshScalingDel4"][:ne] * h_mom_eddy_visc4
            r_dc4 = (u_mix * del4u_div * inv_dc[:ne])[:, None]
            r_dv4 = (u_mix * np.minimum(inv_dv[:ne], 4.0 * inv_dc[:ne]))[:, None]
            u_diff4 = (dsd[e2] - dsd[e1]) * r_dc4 - (dsv[v2] - dsv[v1]) * r_dv4
            tend_u_euler[:ne] = tend_u_euler[:ne] - rho_edge[:ne] * u_diff4
        v_mom = _f(a, "config_v_mom_eddy_visc2")
        if v_mom > 0.0 and nl > 2:  # vertical mixing of u (dyn_tend.py:2730-2780), full state
            zg = a["zgrid"]
            zi = lambda k0, k1: 0.5 * (zg[e1, k0:k1] + zg[e2, k0:k1])
            z1, z2, z3, z4 = zi(0, nl - 2), zi(1, nl - 1), zi(2, nl), zi(3, nl + 1)
            zm, z0, zp = 0.5 * (z1 + z2), 0.5 * (z2 + z3), 0.5 * (z3 + z4)
            uu = u[:ne]
            if not bool(a.get("config_mix_full", True)):  # perturbation from the initial profile
                ang = a["angleEdge"][:ne, None]
                uu = uu - a["u_init"][None, :nl] * np.cos(ang) - a["v_init"][None, :nl] * np.sin(ang)
            tend_u_euler[:ne, 1:nl - 1] = tend_u_euler[:ne, 1:nl - 1] + rho_edge[:ne, 1:nl - 1] * v_mom * (
                (uu[:, 2:nl] - uu[:, 1:nl - 1]) / (zp - z0) - (uu[:, 1:nl - 1] - uu[:, :nl - 2]) / (z0 - zm)
            ) / (0.5 * (zp - zm))
    if bool(a.get("config_rayleigh_damp_u", False)):  # top-level damping of u, every RK stage
        nray = _i(a, "config_number_rayleigh_damp_u_levels")  # (dyn_tend.py:10066-10072, 2956-2990)
        coef = 1.0 / (float(nray) * (_f(a, "config_rayleigh_damp_u_timescale_days") * 86400.0))
        k0 = nl - nray
        damp = ((np.arange(k0, nl, dtype=np.float64) + 1.0) - float(k0)) * coef
        tend_u[:, k0:] = tend_u[:, k0:] - rho_edge[:ne, k0:] * u[:ne, k0:] * damp[None, :]
    tend_u = zpad(tend_u + tend_u_euler[:ne])

    # ---- w tendency ----
    adv = idx0(a["advCellsForEdge"][:ne], nc)
    n_adv = np.asarray(a["nAdvCellsForEdge"][:ne]).astype(np.int64)
    acoef, acoef3 = a["adv_coefs"][:ne], a["adv_coefs_3rd"][:ne]
    tw = np.zeros((nc, nl + 1))
    for j, valid, e in slots():
        ru_w = fzm[1:] * ru[e, 1:nl] + fzp[1:] * ru[e, :nl - 1]
        fl = None
        for m in range(adv.shape[1]):
            vm = m < n_adv[e]
            cell = np.where(vm, adv[e, m], 0)
            sw = acoef[e, m][:, None] + _sgn(ru_w) * acoef3[e, m][:, None]
            c = np.where(vm[:, None], sw * w[cell, 1:nl], 0.0)
            fl = c if fl is None else fl + c
        tw[:, 1:nl] = tw[:, 1:nl] - np.where(valid[:, None], sign[:, j, None] * ru_w * fl, 0.0)
    if rk_step == 1:
        tend_w_euler = np.zeros((nc + 1, nl + 1))
        delsq_w = np.zeros((nc + 1, nl + 1))
        for j, valid, e in slots():
            es = np.where(valid, 0.5 * inv_area[:nc] * sign[:, j] * dv[e] * inv_dc[e], 0.0)[:, None]
            c1, c2 = e1[e], e2[e]
            flux = es * (rho_edge[e, 1:nl] + rho_edge[e, :nl - 1]) * (w[c2, 1:nl] - w[c1, 1:nl])
            delsq_w[:nc, 1:nl] = delsq_w[:nc, 1:nl] + flux
            flux = flux * a["meshScalingDel2"][e][:, None] * 0.25 * \
                (kdiff[c1, 1:nl] + kdiff[c2, 1:nl] + kdiff[c1, :nl - 1] + kdiff[c2, :nl - 1])
            tend_w_euler[:nc, 1:nl] = tend_w_euler[:nc, 1:nl] + flux
        if h_mom_eddy_visc4 > 0.0:
            for j, valid, e in slots():
                es = np.where(valid, a["meshScalingDel4"][e] * (h_mom_eddy_visc4 * inv_area[:nc]) * dv[e]
                              * sign[:, j] * inv_dc[e], 0.0)[:, None]
                c1, c2 = e1[e], e2[e]
                tend_w_euler[:nc, 1:nl] = tend_w_euler[:nc, 1:nl] - es * (delsq_w[c2, 1:nl] - delsq_w[c1, 1:nl])
    else:
        tend_w_euler = a["tend_w_euler_in"].copy()
    wdwz = np.zeros((nc, nl + 1))
    rwc = rw[:nc]
    wc = w[:nc]
    wdwz[:, 1] = 0.25 * (rwc[:, 1] + rwc[:, 0]) * (wc[:, 1] + wc[:, 0])
    for k in range(2, nl - 1):
        wdwz[:, k] = flux3(wc[:, k - 2], wc[:, k - 1], wc[:, k], wc[:, k + 1], 0.5 * (rwc[:, k] + rwc[:, k - 1]), 1.0)
    k = nl - 1
    wdwz[:, k] = 0.25 * (rwc[:, k] + rwc[:, k - 1]) * (wc[:, k] + wc[:, k - 1])
    tw[:, 1:nl] = tw[:, 1:nl] * inv_area[:nc, None] - rdzu[None, 1:] * (wdwz[:, 2:] - wdwz[:, 1:nl])
    if rk_step == 1:
        cqw = a["cqw"]
        tend_w_euler[:nc, 1:nl] = tend_w_euler[:nc, 1:nl] - cqw[:nc, 1:nl] * (
            rdzu[None, 1:] * (pp[:nc, 1:] - pp[:nc, :nl - 1])
            - (fzm[None, 1:] * dpdz[:nc, 1:] + fzp[None, 1:] * dpdz[:nc, :nl - 1]))
        v_mom = _f(a, "config_v_mom_eddy_visc2")
        if v_mom > 0.0:  # vertical mixing of w (dyn_tend.py:4636-4648)
            rz = a["rho_zz"][:nc]
            rho_half = 0.5 * (rz[:, 1:nl] + rz[:, :nl - 1])
            w_up = (wc[:, 2:nl + 1] - wc[:, 1:nl]) * rdzw[1:nl]
            w_down = (wc[:, 1:nl] - wc[:, :nl - 1]) * rdzw[:nl - 1]
            tend_w_euler[:nc, 1:nl] = tend_w_euler[:nc, 1:nl] + v_mom * rho_half * (w_up - w_down) * rdzu[1:nl]
    tw[:, 1:nl] = tw[:, 1:nl] + tend_w_euler[:nc, 1:nl]
    tend_w = zpad(tw)

    # ---- theta tendency ----
    tt = None
    for j, valid, e in slots():
        fl = None
        for m in range(adv.shape[1]):
            vm = m < n_adv[e]
            cell = np.where(vm, adv[e, m], 0)
            sw = acoef[e, m][:, None] + _sgn(ru[e]) * acoef3[e, m][:, None]
            c = np.where(vm[:, None], sw * theta_m[cell], 0.0)
            fl = c if fl is None else fl + c
        c = -np.where(valid[:, None], sign[:, j, None] * ru[e] * fl, 0.0)
        tt = c if tt is None else tt + c
    if rk_step > 1:
        th_s = a["theta_m_save"]
        ru_s = a["ru_save"]
        for j, valid, e in slots():
            flux = np.where(valid, sign[:, j] * dv[e], 0.0)[:, None] * (ru_s[e] - ru[e]) * 0.5 * \
                (th_s[e2[e]] + th_s[e1[e]])
            tt = tt - flux
    if rk_step == 1:
        tend_theta_euler = np.zeros((nc + 1, nl))
        delsq_t = np.zeros((nc + 1, nl))
        for j, valid, e in slots():
            es = np.where(valid, inv_area[:nc] * sign[:, j] * dv[e] * inv_dc[e], 0.0)[:, None]
            pr = (prandtl_inv * a["meshScalingDel2"][e])[:, None]
            c1, c2 = e1[e], e2[e]
            flux = es * (theta_m[c2] - theta_m[c1]) * rho_edge[e]
            delsq_t[:nc] = delsq_t[:nc] + flux
            flux = flux * 0.5 * (kdiff[c1] + kdiff[c2]) * pr
            tend_theta_euler[:nc] = tend_theta_euler[:nc] + flux
        if h_theta_eddy_visc4 > 0.0:
            for j, valid, e in slots():
                es = np.where(valid, a["meshScalingDel4"][e] * (h_theta_eddy_visc4 * prandtl_inv * inv_area[:nc])
                              * dv[e] * sign[:, j] * inv_dc[e], 0.0)[:, None]
                c1, c2 = e1[e], e2[e]
                tend_theta_euler[:nc] = tend_theta_euler[:nc] - es * (delsq_t[c2] - delsq_t[c1])
        v_th = _f(a, "config_v_theta_eddy_visc2")
        if v_th > 0.0 and nl > 2:  # vertical mixing of theta (dyn_tend.py:5064-5100), full state
            zg = a["zgrid"][:nc]
            z1, z2, z3, z4 = zg[:, 0:nl - 2], zg[:, 1:nl - 1], zg[:, 2:nl], zg[:, 3:nl + 1]
            zm, z0, zp = 0.5 * (z1 + z2), 0.5 * (z2 + z3), 0.5 * (z3 + z4)
            th = theta_m[:nc]
            if not bool(a.get("config_mix_full", True)):
                th = th - a["t_init"][:nc]
            diff = (th[:, 2:nl] - th[:, 1:nl - 1]) / (zp - z0) - (th[:, 1:nl - 1] - th[:, :nl - 2]) / (z0 - zm)
            tend_theta_euler[:nc, 1:nl - 1] = tend_theta_euler[:nc, 1:nl - 1] + \
                v_th * prandtl_inv * a["rho_zz"][:nc, 1:nl - 1] * diff / (0.5 * (zp - zm))
    else:
        tend_theta_euler = a["tend_theta_euler_in"].copy()
    th = theta_m[:nc]
    th_s = a["theta_m_save"][:nc]
    rws = a["rw_save"][:nc]
    wdtz = np.zeros((nc, nl + 1))
    k = 1
    wdtz[:, k] = rwc[:, k] * (fzm[k] * th[:, k] + fzp[k] * th[:, k - 1])
    wdtz[:, k] = wdtz[:, k] + (rws[:, k] - rwc[:, k]) * (fzm[k] * th_s[:, k] + fzp[k] * th_s[:, k - 1])
    for k in range(2, nl - 1):
        wdtz[:, k] = flux3(th[:, k - 2], th[:, k - 1], th[:, k], th[:, k + 1], rwc[:, k], coef3)
        wdtz[:, k] = wdtz[:, k] + (rws[:, k] - rwc[:, k]) * (fzm[k] * th_s[:, k] + fzp[k] * th_s[:, k - 1])
    k = nl - 1
    wdtz[:, k] = rws[:, k] * (fzm[k] * th[:, k] + fzp[k] * th[:, k - 1])
    rho_zz = a["rho_zz"][:nc]
    rtd = a["rt_diabatic_tend"][:nc]
    tt = tt * inv_area[:nc, None] - rdzw[None, :] * (wdtz[:, 1:] - wdtz[:, :nl])
    rthdynten = (tt - tend_rho[:nc] * th) / rho_zz
    tt = tt + rho_zz * rtd
    tt = tt + tend_theta_euler[:nc]
    return {"tend_u": tend_u, "tend_rho": tend_rho, "tend_theta": zpad(tt), "tend_w": tend_w,
            "tend_u_euler": tend_u_euler, "tend_w_euler": tend_w_euler,
            "tend_theta_euler": tend_theta_euler, "h_divergence": h_div_p, "kdiff": kdiff,
            "rthdynten": zpad(rthdynten)}


# --------------------------------------------------------------------------------------
# scalar transport  (dynamics/advance_scalars.py:1272, composition :861, Pattern-C
# pattern_c.py:234-305; monotone: dynamics/advance_scalars_mono.py:3332, tile :1476,
# neighbour bounds autodiff/soft_limiter.py:72)
# --------------------------------------------------------------------------------------

def _pattern_c(a, sfield, uh, ne, nc):
    """Edge high-order value sum_m (adv_coefs + sign(uh) adv_coefs_3rd) q[advCell_m]."""
    adv = idx0(a["advCellsForEdge"][:ne], nc)
    n_adv = np.asarray(a["nAdvCellsForEdge"][:ne]).astype(np.int64)
    acoef, acoef3 = a["adv_coefs"][:ne], a["adv_coefs_3rd"][:ne]
    sg = _sgn(uh[:ne])
    out = None
    for m in range(adv.shape[1]):
        vm = m < n_adv
        cell = np.where(vm, adv[:, m], nc)
        wgt = acoef[:, m, None] + sg * acoef3[:, m, None]
        c = wgt[:, :, None] * sfield[cell]
        c = np.where(vm[:, None, None], c, 0.0)
        out = c if out is None else out + c
    return out


def _time_weights(advance_density, rk_step, order):
    if advance_density == 0:
        w_new = 1.0
    elif rk_step == 1 and order == 3:
        w_new = 1.0 / 3.0
    elif (rk_step == 1 and order == 2) or rk_step == 2:
        w_new = 1.0 / 2.0
    else:
        w_new = 1.0
    return 1.0 - w_new, w_new


def advance_scalars(a):
    """Explicit flux-form RK-stage scalar update (non-monotone)."""
    nc, ne, nl = _i(a, "nCells"), _i(a, "nEdges"), _i(a, "nVertLevels")
    dt, coef3 = _f(a, "dt"), _f(a, "coef_3rd_order")
    w_old, w_new = _time_weights(_i(a, "advance_density"), _i(a, "rk_step"),
                                 _i(a, "config_time_integration_order"))
    s_new = a["scalar_new"]
    s_old = a["scalar_old"]
    uh = a["uhAvg"]
    ww = a["wwAvg"][:nc]
    sn_pad = s_new.copy()
    sn_pad[nc] = 0.0
    hf = _pattern_c(a, sn_pad, uh, ne, nc)
    eoc = idx0(a["edgesOnCell"][:nc], ne)
    n_eoc = np.asarray(a["nEdgesOnCell"][:nc]).astype(np.int64)
    sign = a["edgesOnCell_sign"][:nc]
    div = None
    for j in range(eoc.shape[1]):
        valid = (j < n_eoc) & (eoc[:, j] < ne)
        e = np.where(valid, eoc[:, j], 0)
        c = (-sign[:, j, None] * uh[e])[:, :, None] * hf[e]
        c = np.where(valid[:, None, None], c, 0.0)
        div = c if div is None else div + c
    tend_save = np.zeros_like(a["scalar_tend_save"][:nc]) if not a.get("do_physics", False) \
        else a["scalar_tend_save"][:nc]
    tend_col = div * a["invAreaCell"][:nc, None, None] + tend_save
    fnm, fnp, rdnw = a["fnm"][:nl], a["fnp"][:nl], a["rdnw"][:nl]
    sn = s_new[:nc]
    wdtn = np.zeros((nc, nl + 1, sn.shape[2]))
    wdtn[:, 1] = ww[:, 1:2] * (fnm[1] * sn[:, 1] + fnp[1] * sn[:, 0])
    for k in range(2, nl - 1):
        wdtn[:, k] = flux3(sn[:, k - 2], sn[:, k - 1], sn[:, k], sn[:, k + 1], ww[:, k:k + 1], coef3)
    k = nl - 1
    wdtn[:, k] = ww[:, k:k + 1] * (fnm[k] * sn[:, k] + fnp[k] * sn[:, k - 1])
    vdiv = rdnw[None, :, None] * (wdtn[:, 1:] - wdtn[:, :nl])
    rho_old = a["rho_zz_old"][:nc]
    rho_i = w_old * rho_old + w_new * a["rho_zz_new"][:nc]
    out = s_new.copy()
    out[:nc] = (s_old[:nc] * rho_old[:, :, None] + dt * (tend_col - vdiv)) * (1.0 / rho_i)[:, :, None]
    hfa = a["horiz_flux_arr"].copy()
    hfa[:ne] = hf
    tso = a["scalar_tend_save"].copy()
    tso[:nc] = tend_save
    return {"scalar_new": out, "scalar_tend_save": tso, "horiz_flux_arr": hfa}


def advance_scalars_mono(a):
    """Monotone (flux-corrected) scalar update for the final transport RK stage."""
    nc, ne, nl = _i(a, "nCells"), _i(a, "nEdges"), _i(a, "nVertLevels")
    dt, coef3 = _f(a, "dt"), _f(a, "coef_3rd_order")
    eps = 1.0e-20
    uh = a["uhAvg"]
    ww = a["wwAvg"][:nc]
    rho_old = a["rho_zz_old"][:nc]
    fnm, fnp, rdnw = a["fnm"][:nl], a["fnp"][:nl], a["rdnw"][:nl]
    dv = a["dvEdge"]
    inv_area = a["invAreaCell"][:nc]
    eoc = idx0(a["edgesOnCell"][:nc], ne)
    n_eoc = np.asarray(a["nEdgesOnCell"][:nc]).astype(np.int64)
    sign = a["edgesOnCell_sign"][:nc]
    coe = idx0(a["cellsOnEdge"][:ne], nc)
    e1, e2 = coe[:, 0], coe[:, 1]

    scalars_old = a["scalars_old"].copy()
    scalars_old[:nc] = scalars_old[:nc] + dt * a["scalar_tend"][:nc] / rho_old[:, :, None]
    scalars_new_in = a["scalars_new"]

    # density at the end of the stage from the averaged mass fluxes
    hdiv = None
    for j in range(eoc.shape[1]):
        valid = (j < n_eoc) & (eoc[:, j] < ne)
        e = np.where(valid, eoc[:, j], 0)
        c = (uh[e] * (-sign[:, j] * dv[e])[:, None]) * np.where(valid, inv_area, 0.0)[:, None]
        hdiv = c if hdiv is None else hdiv + c
    vdiv = rdnw[None, :] * (ww[:, 1:nl + 1] - ww[:, :nl])
    rho_int = rho_old + dt * (hdiv - vdiv)

    so_all = scalars_old.copy()
    so_all[nc] = 0.0
    sn_all = scalars_new_in.copy()
    sn_all[nc] = 0.0
    so = so_all[:nc]
    sn = sn_all[:nc]
    ns = so.shape[2]
    smax = np.empty((nc, nl, ns))
    smin = np.empty((nc, nl, ns))
    smax[:, 0] = np.maximum(so[:, 0], so[:, 1])
    smin[:, 0] = np.minimum(so[:, 0], so[:, 1])
    for k in range(1, nl - 1):
        smax[:, k] = np.maximum(np.maximum(so[:, k - 1], so[:, k]), so[:, k + 1])
        smin[:, k] = np.minimum(np.minimum(so[:, k - 1], so[:, k]), so[:, k + 1])
    smax[:, nl - 1] = np.maximum(so[:, nl - 1], so[:, nl - 2])
    smin[:, nl - 1] = np.minimum(so[:, nl - 1], so[:, nl - 2])
    wdtn = np.zeros((nc, nl + 1, ns))
    wdtn[:, 1] = ww[:, 1:2] * (fnm[1] * sn[:, 1] + fnp[1] * sn[:, 0])
    for k in range(2, nl - 1):
        wdtn[:, k] = flux3(sn[:, k - 2], sn[:, k - 1], sn[:, k], sn[:, k + 1], ww[:, k:k + 1], coef3)
    k = nl - 1
    wdtn[:, k] = ww[:, k:k + 1] * (fnm[k] * sn[:, k] + fnp[k] * sn[:, k - 1])
    coc = idx0(a["cellsOnCell"][:nc], nc)
    nmax = None
    nmin = None
    for j in range(coc.shape[1]):
        valid = (j < n_eoc) & (coc[:, j] < nc)
        val = so_all[coc[:, j]]
        vm = valid[:, None, None]
        if nmax is None:
            nmax = np.where(vm, val, -np.finfo(np.float64).max)
            nmin = np.where(vm, val, np.finfo(np.float64).max)
            seen = valid.copy()
        else:
            comb = (valid & seen)[:, None, None]
            repl = (valid & ~seen)[:, None, None]
            nmax = np.where(comb, np.maximum(nmax, val), np.where(repl, val, nmax))
            nmin = np.where(comb, np.minimum(nmin, val), np.where(repl, val, nmin))
            seen = seen | valid
    smax = np.maximum(smax, nmax)
    smin = np.minimum(smin, nmin)

    # high-order and upwind fluxes
    flux_edge = uh[:ne, :, None] * _pattern_c(a, sn_all, uh, ne, nc)
    wmid = ww[:, 1:nl, None]
    flux_up_mid = dt * (wmid * np.where(wmid >= 0.0, so[:, :nl - 1], so[:, 1:nl]))
    rows = so * rho_old[:, :, None]
    rows[:, :nl - 1] = rows[:, :nl - 1] - flux_up_mid * rdnw[None, :nl - 1, None]
    rows[:, 1:nl] = rows[:, 1:nl] + flux_up_mid * rdnw[None, 1:nl, None]
    wmid_flux = dt * wdtn[:, 1:nl] - flux_up_mid
    mz = lambda x: np.maximum(x, 0.0)
    prev = np.concatenate([wdtn[:, 0:1], wmid_flux], axis=1)
    nxt = np.concatenate([wmid_flux, wdtn[:, nl:nl + 1]], axis=1)
    r = rdnw[None, :, None]
    scale_in = -r * ((-mz(-nxt)) - mz(prev))
    scale_out = -r * (mz(nxt) - (-mz(-prev)))
    up = uh[:ne, :, None]
    flux_up_edge = dv[:ne, None, None] * dt * (up * np.where(up >= 0.0, so_all[e1], so_all[e2]))
    flux_tmp = dt * flux_edge - flux_up_edge
    for j in range(eoc.shape[1]):
        valid = (j < n_eoc) & (eoc[:, j] < ne)
        e = np.where(valid, eoc[:, j], 0)
        vw = np.where(valid, inv_area, 0.0)
        sw = sign[:, j] * vw
        rows = rows - flux_up_edge[e] * sw[:, None, None]
        sf = sign[:, j, None, None] * flux_tmp[e]
        scale_out = scale_out - mz(sf) * vw[:, None, None]
        scale_in = scale_in - (-mz(-sf)) * vw[:, None, None]
    rint = rho_int[:, :, None]
    sc_in = np.clip((smax * rint - rows) / (scale_in + eps), 0.0, 1.0)
    sc_out = np.clip((smin * rint - rows) / (scale_out - eps), 0.0, 1.0)
    pad3 = lambda x: np.concatenate([x, np.zeros((1,) + x.shape[1:])])
    sc_in_p, sc_out_p = pad3(sc_in), pad3(sc_out)
    fl = flux_tmp
    lim = np.where(fl >= 0.0, np.minimum(sc_out_p[e1], sc_in_p[e2]), np.minimum(sc_in_p[e1], sc_out_p[e2]))
    flux_lim = fl * lim
    wl = wmid_flux * np.where(wmid_flux >= 0.0, np.minimum(sc_out[:, :nl - 1], sc_in[:, 1:nl]),
                              np.minimum(sc_out[:, 1:nl], sc_in[:, :nl - 1]))
    wl_full = np.concatenate([wdtn[:, 0:1], wl, wdtn[:, nl:nl + 1]], axis=1)
    vdelta = wl_full[:, 1:] - wl_full[:, :nl]
    for j in range(eoc.shape[1]):
        valid = (j < n_eoc) & (eoc[:, j] < ne)
        e = np.where(valid, eoc[:, j], 0)
        sw = sign[:, j] * np.where(valid, inv_area, 0.0)
        rows = rows - flux_lim[e] * sw[:, None, None]
    stage2 = (rows - rdnw[None, :, None] * vdelta) / rint
    out = scalars_new_in.copy()
    out[:nc] = np.maximum(stage2, 0.0)
    return {"scalars_new": out, "scalars_old": scalars_old, "rho_zz_int": pad3(rho_int)[:, :]}


def surface_pressure(nCells, rho_zz, zz, qv, pressure_p, pressure_base, zgrid, gravity=GRAVITY):
    """Hydrostatic surface pressure of the MPAS physics interface
    (mpas_pytorch/diagnostics.py:10, formula :77-82): per active cell, with the padding
    row (when given) set to zero."""
    c = int(nCells)
    tem1 = zgrid[:c, 1] - zgrid[:c, 0]
    tem2 = zgrid[:c, 2] - zgrid[:c, 1]
    rho1 = rho_zz[:c, 0] * zz[:c, 0] * (1.0 + qv[:c, 0])
    rho2 = rho_zz[:c, 1] * zz[:c, 1] * (1.0 + qv[:c, 1])
    hyd = 0.5 * gravity * tem1 * (rho1 - 0.5 * (rho2 - rho1) * tem1 / (tem1 + tem2))
    sp = hyd + pressure_p[:c, 0] + pressure_base[:c, 0]
    if rho_zz.shape[0] == c + 1:
        sp = np.concatenate([sp, np.zeros(1)])
    return sp
