"""Oracle (test infrastructure): numpy restatement of the reverse mode (vector-Jacobian
products) of the reference's dynamics stages and of the whole large step.

The reference differentiates its stages with torch autograd (``atm_srk3(differentiable=
True)``, mpas_pytorch/dynamics/time_integration.py:4897-4948) through the custom Functions
of ``dynamics/dyn_tend.py:1194,1413,1568,3860``, ``autodiff/tridiagonal_solve.py:232-291``
and ``autodiff/tridiagonal_factor.py:183-231``; hard branches (the sign selectors of the
third-order fluxes, ``abs``, ``min``) carry the derivative of the branch taken, as the
reference's AD control domain states (``autodiff/soft_limiter.py:1-10``).  Each function
here takes the stage's keyword arguments ``a`` (the same mapping the forward restatements
in ``stages.py`` take, with the reference's keyword names) and the cotangents ``g`` of the
stage outputs (reference output names; a missing name is a zero cotangent), and returns
the cotangents of the stage's floating-point inputs.  Transposed stencils are written as
scatters (``np.add.at``); the CUDA kernels use the equivalent deterministic gathers.

Scope (the configurations the dynamics derivative supports): dry columns
(``moist_end < moist_start``), flat or terrain-following levels (the slope terms'
upwind selections held fixed), horizontal mixing ``2d_smagorinsky`` or ``2d_fixed``
with or without the del4 filter, vertical mixing, CAM and Rayleigh damping; any RK
order, substep and split counts.

This module is test infrastructure: only ``tests/`` read it.
"""

from __future__ import annotations

import numpy as np

from . import adjoint as A
from . import stages as S

GRAVITY, RGAS, CP, P0 = S.GRAVITY, S.RGAS, S.CP, S.P0
PRE = "_vertical_implicit_coefficients_"

__all__ = ["vimp_vjp", "acoustic_vjp", "divdamp_vjp", "smlstep_vjp", "recover_vjp", "diag_vjp",
           "dyn_tend_vjp", "flux3_grads"]


def _i(a, k):
    return S._i(a, k)


def _f(a, k):
    return S._f(a, k)


def _z(x):
    return np.zeros_like(x, dtype=np.float64)


def _g(g, k, like):
    v = g.get(k)
    return np.zeros_like(like, dtype=np.float64) if v is None else np.asarray(v, dtype=np.float64)


def _add(out, k, v):
    out[k] = out[k] + v if k in out else v


def _sgn(x):
    return np.where(x < 0.0, -1.0, 1.0)


def _absgrad(x):
    """d|x|/dx as torch takes it: sign(x), 0 at 0."""
    return np.sign(x)


def flux3_grads(qm2, qm1, q0, qp1, ua, c3):
    """Partial derivatives of flux3 (dyn_tend.py:839,853) with respect to its six
    arguments (qm2, qm1, q0, qp1, ua); |ua| differentiated as sign(ua)."""
    au = np.abs(ua)
    s = _absgrad(ua)
    d_qm2 = (-ua - c3 * au) / 12.0
    d_qm1 = (7.0 * ua + 3.0 * c3 * au) / 12.0
    d_q0 = (7.0 * ua - 3.0 * c3 * au) / 12.0
    d_qp1 = (-ua + c3 * au) / 12.0
    d_ua = ((7.0 * (q0 + qm1) - (qp1 + qm2)) + c3 * s * ((qp1 - qm2) - 3.0 * (q0 - qm1))) / 12.0
    return d_qm2, d_qm1, d_q0, d_qp1, d_ua


# --------------------------------------------------------------------------------------
# vertical implicit coefficients (vert_imp_coefs.py:188) and the Thomas factor
# --------------------------------------------------------------------------------------

def vimp_vjp(a, g):
    """Cotangents of p (exner), t (theta_m) and rt (rtheta_p) from those of cofwz, coftz,
    cofwt, a_tri, alpha_tri and gamma_tri (cofrz and cofwr depend on the mesh only)."""
    nc, nl = _i(a, "nCells"), _i(a, "nVertLevels")
    dts, epssm = _f(a, "dts"), _f(a, "epssm")
    g0, rgas, cp = _f(a, "gravity"), _f(a, "rgas"), _f(a, "cp")
    dtseps = 0.5 * dts * (1.0 + epssm)
    rcv = rgas / (cp - rgas)
    c2 = cp * rcv
    rdzw, fzm, fzp, rdzu = (a[k][:nl] for k in ("rdzw", "fzm", "fzp", "rdzu"))
    zz, cqw, p, t, rb, rtb, pb, rt, qtot = (a[k][:nc, :nl] for k in
                                             ("zz", "cqw", "p", "t", "rb", "rtb", "pb", "rt", "qtot"))
    fw = S.vert_imp_coefs(a)
    cofrz = fw["cofrz"]
    cofwr, cofwz, coftz, cofwt = (fw[PRE + k] for k in ("cofwr_active", "cofwz_active", "coftz_active",
                                                       "cofwt_active"))
    a_tri, alpha, gamma = (fw[PRE + k] for k in ("a_tri_active", "alpha_tri_active", "gamma_tri_active"))
    c_tri = np.zeros((nc, nl))
    c_tri[:, 1:] = (-cofwz[:, 1:] * coftz[:, 2:nl + 1] * rdzw[1:] * zz[:, 1:] - cofwr[:, 1:] * cofrz[1:]
                    + cofwt[:, 1:] * coftz[:, 2:nl + 1] * rdzw[1:])
    g_alpha = _g(g, PRE + "alpha_tri_active", alpha)
    g_gamma = _g(g, PRE + "gamma_tri_active", gamma)
    ga, gb, gc = A.factor_vjp(a_tri, c_tri, alpha, gamma, g_alpha, g_gamma)
    ga = ga + _g(g, PRE + "a_tri_active", a_tri)
    g_wz = _g(g, PRE + "cofwz_active", cofwz).copy()
    g_tz = _g(g, PRE + "coftz_active", coftz).copy()
    g_wt = _g(g, PRE + "cofwt_active", cofwt).copy()
    for k in range(1, nl):
        # a_tri[k] = -cofwz_k coftz_(k-1) rdzw_(k-1) zz_(k-1) + cofwr cofrz - cofwt_(k-1) coftz_(k-1) rdzw_(k-1)
        ak = ga[:, k]
        g_wz[:, k] += ak * (-coftz[:, k - 1] * rdzw[k - 1] * zz[:, k - 1])
        g_tz[:, k - 1] += ak * (-cofwz[:, k] * rdzw[k - 1] * zz[:, k - 1] - cofwt[:, k - 1] * rdzw[k - 1])
        g_wt[:, k - 1] += ak * (-coftz[:, k - 1] * rdzw[k - 1])
        # b_tri[k]
        bk = gb[:, k]
        s = rdzw[k] * zz[:, k] + rdzw[k - 1] * zz[:, k - 1]
        g_wz[:, k] += bk * coftz[:, k] * s
        g_tz[:, k] += bk * (cofwz[:, k] * s - (cofwt[:, k] * rdzw[k] - cofwt[:, k - 1] * rdzw[k - 1]))
        g_wt[:, k] += bk * (-coftz[:, k] * rdzw[k])
        g_wt[:, k - 1] += bk * (coftz[:, k] * rdzw[k - 1])
        # c_tri[k]
        ck = gc[:, k]
        g_wz[:, k] += ck * (-coftz[:, k + 1] * rdzw[k] * zz[:, k])
        g_tz[:, k + 1] += ck * (-cofwz[:, k] * rdzw[k] * zz[:, k] + cofwt[:, k] * rdzw[k])
        g_wt[:, k] += ck * (coftz[:, k + 1] * rdzw[k])
    gp = np.zeros((nc, nl))
    gt = np.zeros((nc, nl))
    grt = np.zeros((nc, nl))
    z_i = fzm[1:] * zz[:, 1:] + fzp[1:] * zz[:, :-1]
    fac = dtseps * c2 * z_i * rdzu[1:nl] * cqw[:, 1:]
    gp[:, 1:] += g_wz[:, 1:] * fac * fzm[1:]
    gp[:, :-1] += g_wz[:, 1:] * fac * fzp[1:]
    gt[:, 1:] += g_tz[:, 1:nl] * dtseps * fzm[1:]
    gt[:, :-1] += g_tz[:, 1:nl] * dtseps * fzp[1:]
    x = 0.5 * dtseps * rcv * zz * g0 * rb / (1.0 + qtot)
    den = (rtb + rt) * pb
    gp += g_wt * x / den
    grt += g_wt * (-x * p * pb / (den * den))
    out = {}
    for k, v in (("p", gp), ("t", gt), ("rt", grt)):
        full = np.zeros_like(a[k], dtype=np.float64)
        full[:nc, :nl] = v
        out[k] = full
    return out


# --------------------------------------------------------------------------------------
# acoustic substep (acoustic_step.py:1297)
# --------------------------------------------------------------------------------------

def acoustic_vjp(a, g):
    nc, ne, nl = _i(a, "nCells"), _i(a, "nEdges"), _i(a, "nVertLevels")
    small = _i(a, "small_step")
    first = small == 1
    dts, epssm, resm, c2 = _f(a, "dts"), _f(a, "epssm"), _f(a, "resm"), _f(a, "c2")
    coe = S.idx0(a["cellsOnEdge"][:ne], nc)
    e1, e2 = coe[:, 0], coe[:, 1]
    zz_f, exner = a["zz"], a["exner"]
    rtpp, rpp = a["rtheta_pp"], a["rho_pp"]
    inv_dc = a["invDcEdge"][:ne, None]
    mask = (1.0 - a["specZoneMaskEdge"][:ne, None])
    cqu = a["cqu"][:ne]
    # ---- forward recomputation
    if not first:
        d = (rtpp[e2] - rtpp[e1]) * inv_dc
        den = 0.5 * (zz_f[e2] + zz_f[e1])
        pg1 = d / den
        exs = exner[e1] + exner[e2]
        ru_p_new = a["ru_p"][:ne] + dts * (a["tend_ru"][:ne] - mask * (cqu * 0.5 * c2 * exs * pg1
                                                                       + 0.5 * a["zxu"][:ne] * GRAVITY * (rpp[e1] + rpp[e2])))
    else:
        ru_p_new = dts * a["tend_ru"][:ne]
    fw = S.acoustic_step(a)
    cofrz = a["cofrz"][:nl]
    rdzw = a["rdzw"][:nl]
    coftz, cofwz, cofwr, cofwt = (a[PRE + k] for k in ("coftz_active", "cofwz_active", "cofwr_active",
                                                      "cofwt_active"))
    a_tri, alpha, gamma = (a[PRE + k] for k in ("a_tri_active", "alpha_tri_active", "gamma_tri_active"))
    zz = zz_f[:nc, :nl]
    th = a["theta_m"]
    eoc = S.idx0(a["edgesOnCell"][:nc], ne)
    n_eoc = np.asarray(a["nEdgesOnCell"][:nc]).astype(np.int64)
    sign = a["edgesOnCell_sign"][:nc]
    inv_area = a["invAreaCell"][:nc]
    dv = a["dvEdge"]
    rho_in = np.zeros((nc, nl)) if first else rpp[:nc].copy()
    rt_in = np.zeros((nc, nl)) if first else rtpp[:nc].copy()
    rwp = np.zeros((nc, nl + 1)) if first else a["rw_p"][:nc].copy()
    slots = []
    rs = np.zeros((nc, nl))
    ts = np.zeros((nc, nl))
    for j in range(eoc.shape[1]):
        valid = (j < n_eoc) & (eoc[:, j] < ne)
        e = np.where(valid, eoc[:, j], 0)
        wj = np.where(valid, sign[:, j] * dv[e], 0.0)
        flux = dts * wj[:, None] * ru_p_new[e] * inv_area[:, None]
        th_e = 0.5 * (th[e2[e]] + th[e1[e]])
        slots.append((valid, e, wj, flux, th_e))
        rs = rs - flux * valid[:, None]
        ts = ts - flux * th_e * valid[:, None]
    rs = rho_in + dts * a["tend_rho"][:nc] + rs - cofrz[None, :] * resm * (rwp[:, 1:] - rwp[:, :nl])
    ts = (rt_in + dts * a["tend_rt"][:nc] + ts
          - resm * rdzw[None, :] * (coftz[:, 1:] * rwp[:, 1:] - coftz[:, :nl] * rwp[:, :nl]))
    rhs = rwp.copy()
    rhs[:, 1:nl] = (rwp[:, 1:nl] + dts * a["tend_rw"][:nc, 1:nl]
                    - cofwz[:, 1:] * ((zz[:, 1:] * ts[:, 1:] - zz[:, :-1] * ts[:, :-1])
                                      + resm * (zz[:, 1:] * rt_in[:, 1:] - zz[:, :-1] * rt_in[:, :-1]))
                    - cofwr[:, 1:] * ((rs[:, 1:] + rs[:, :-1]) + resm * (rho_in[:, 1:] + rho_in[:, :-1]))
                    + cofwt[:, 1:] * (ts[:, 1:] + resm * rt_in[:, 1:])
                    + cofwt[:, :-1] * (ts[:, :-1] + resm * rt_in[:, :-1]))
    sol = S.tridiagonal_solve(a_tri, alpha, gamma, rhs)
    fzm, fzp = a["fzm"][:nl], a["fzp"][:nl]
    zz_i = fzm[1:] * zz[:, 1:] + fzp[1:] * zz[:, :-1]
    rho_zz = a["rho_zz"][:nc, :nl]
    rho_i = fzm[1:] * rho_zz[:, 1:] + fzp[1:] * rho_zz[:, :-1]
    dss = a["dss"][:nc, :nl]
    D = 1.0 + dts * dss[:, 1:]
    sol2 = fw["rw_p"][:nc]
    # ---- reverse
    out = {}
    g_sol2 = _g(g, "rw_p", a["rw_p"])[:nc].copy()
    g_ww2 = _g(g, "wwAvg", a["wwAvg"])[:nc].copy()
    g_rho = _g(g, "rho_pp", rpp)[:nc]
    g_rt = _g(g, "rtheta_pp", rtpp)[:nc]
    g_ts = g_rt.copy()
    g_coftz = np.zeros_like(coftz)
    g_coftz[:, 1:] += -g_rt * rdzw[None, :] * sol2[:, 1:]
    g_coftz[:, :nl] += g_rt * rdzw[None, :] * sol2[:, :nl]
    g_sol2[:, 1:] += -g_rt * rdzw[None, :] * coftz[:, 1:]
    g_sol2[:, :nl] += g_rt * rdzw[None, :] * coftz[:, :nl]
    g_rs = g_rho.copy()
    g_sol2[:, 1:] += -g_rho * cofrz[None, :]
    g_sol2[:, :nl] += g_rho * cofrz[None, :]
    g_ww = g_ww2.copy()
    g_sol2[:, 1:nl] += 0.5 * (1.0 + epssm) * g_ww2[:, 1:nl]
    # Rayleigh damping of the solution
    g_sol = g_sol2.copy()
    gs = g_sol2[:, 1:nl] / D
    g_sol[:, 1:nl] = gs
    g_rwd = gs - g_sol2[:, 1:nl]
    w_mid = a["w"][:nc, 1:nl]
    g_rho_i = gs * (-dts * dss[:, 1:] * zz_i * w_mid)
    g_w = np.zeros_like(a["w"], dtype=np.float64)
    g_w[:nc, 1:nl] = gs * (-dts * dss[:, 1:] * zz_i * rho_i)
    g_rw_save = np.zeros_like(a["rw_save"], dtype=np.float64)
    g_rw_save[:nc, 1:nl] = g_rwd
    g_rw = np.zeros_like(a["rw"], dtype=np.float64)
    g_rw[:nc, 1:nl] = -g_rwd
    g_rho_zz = np.zeros_like(a["rho_zz"], dtype=np.float64)
    g_rho_zz[:nc, 1:nl] += fzm[1:] * g_rho_i
    g_rho_zz[:nc, :nl - 1] += fzp[1:] * g_rho_i
    # Thomas solve
    ga, gal, gg, grhs = A.solve_vjp(a_tri, alpha, gamma, rhs, sol, g_sol)
    # right-hand side
    g_rwp = np.zeros((nc, nl + 1))
    g_rt_in = np.zeros((nc, nl))
    g_rho_in = np.zeros((nc, nl))
    r = grhs[:, 1:nl]
    g_rwp[:, 1:nl] += r
    g_tend_rw = np.zeros_like(a["tend_rw"], dtype=np.float64)
    g_tend_rw[:nc, 1:nl] = dts * r
    g_cofwz = np.zeros_like(cofwz)
    g_cofwz[:, 1:] = -r * ((zz[:, 1:] * ts[:, 1:] - zz[:, :-1] * ts[:, :-1])
                           + resm * (zz[:, 1:] * rt_in[:, 1:] - zz[:, :-1] * rt_in[:, :-1]))
    g_ts[:, 1:] += -r * cofwz[:, 1:] * zz[:, 1:]
    g_ts[:, :-1] += r * cofwz[:, 1:] * zz[:, :-1]
    g_rt_in[:, 1:] += -r * cofwz[:, 1:] * resm * zz[:, 1:]
    g_rt_in[:, :-1] += r * cofwz[:, 1:] * resm * zz[:, :-1]
    g_rs[:, 1:] += -r * cofwr[:, 1:]
    g_rs[:, :-1] += -r * cofwr[:, 1:]
    g_rho_in[:, 1:] += -r * cofwr[:, 1:] * resm
    g_rho_in[:, :-1] += -r * cofwr[:, 1:] * resm
    g_cofwt = np.zeros_like(cofwt)
    g_cofwt[:, 1:] += r * (ts[:, 1:] + resm * rt_in[:, 1:])
    g_cofwt[:, :-1] += r * (ts[:, :-1] + resm * rt_in[:, :-1])
    g_ts[:, 1:] += r * cofwt[:, 1:]
    g_rt_in[:, 1:] += r * cofwt[:, 1:] * resm
    g_ts[:, :-1] += r * cofwt[:, :-1]
    g_rt_in[:, :-1] += r * cofwt[:, :-1] * resm
    g_rwp[:, 0] += grhs[:, 0]
    g_rwp[:, nl] += grhs[:, nl]
    # ww accumulation before the solve
    g_ww0 = g_ww.copy()
    g_rwp[:, 1:nl] += 0.5 * (1.0 - epssm) * g_ww[:, 1:nl]
    # ts / rs
    g_rt_in += g_ts
    g_tend_rt = np.zeros_like(a["tend_rt"], dtype=np.float64)
    g_tend_rt[:nc] = dts * g_ts
    g_rwp[:, 1:] += -g_ts * resm * rdzw[None, :] * coftz[:, 1:]
    g_rwp[:, :nl] += g_ts * resm * rdzw[None, :] * coftz[:, :nl]
    g_coftz[:, 1:] += -g_ts * resm * rdzw[None, :] * rwp[:, 1:]
    g_coftz[:, :nl] += g_ts * resm * rdzw[None, :] * rwp[:, :nl]
    g_rho_in += g_rs
    g_tend_rho = np.zeros_like(a["tend_rho"], dtype=np.float64)
    g_tend_rho[:nc] = dts * g_rs
    g_rwp[:, 1:] += -g_rs * cofrz[None, :] * resm
    g_rwp[:, :nl] += g_rs * cofrz[None, :] * resm
    g_ru_p_new = np.zeros((ne + 1, nl))
    g_th = np.zeros_like(th, dtype=np.float64)
    for valid, e, wj, flux, th_e in slots:
        vm = valid[:, None]
        g_flux = np.where(vm, -g_rs - g_ts * th_e, 0.0)
        g_the = np.where(vm, -g_ts * flux, 0.0)
        np.add.at(g_ru_p_new, e, g_flux * (dts * wj[:, None] * inv_area[:, None]))
        np.add.at(g_th, e2[e], 0.5 * g_the)
        np.add.at(g_th, e1[e], 0.5 * g_the)
    g_th[nc] = 0.0
    g_ru_p_new = g_ru_p_new[:ne] + _g(g, "ru_p", a["ru_p"])[:ne] + _g(g, "ruAvg", a["ruAvg"])[:ne]
    g_rpp = np.zeros_like(rpp, dtype=np.float64)
    g_rtpp = np.zeros_like(rtpp, dtype=np.float64)
    g_rw_p = np.zeros_like(a["rw_p"], dtype=np.float64)
    g_wwavg = np.zeros_like(a["wwAvg"], dtype=np.float64)
    g_ru_p = np.zeros_like(a["ru_p"], dtype=np.float64)
    g_ruavg = np.zeros_like(a["ruAvg"], dtype=np.float64)
    g_tend_ru = np.zeros_like(a["tend_ru"], dtype=np.float64)
    g_exner = _g(g, "exner", exner).copy()
    g_w = g_w + _g(g, "w", a["w"])
    g_cqu = np.zeros_like(a["cqu"], dtype=np.float64)
    if not first:
        g_rpp[:nc] += g_rho_in
        g_rtpp[:nc] += g_rt_in
        g_rtpp[:nc] += _g(g, "rtheta_pp_old", a["rtheta_pp_old"])[:nc]
        g_rw_p[:nc] += g_rwp
        g_wwavg[:nc] += g_ww0
        g_ruavg[:ne] += _g(g, "ruAvg", a["ruAvg"])[:ne]
        g_ru_p[:ne] += g_ru_p_new
        g_tend_ru[:ne] += dts * g_ru_p_new
        g_pg = -dts * mask * g_ru_p_new
        np.add.at(g_rpp, e1, g_pg * 0.5 * a["zxu"][:ne] * GRAVITY)
        np.add.at(g_rpp, e2, g_pg * 0.5 * a["zxu"][:ne] * GRAVITY)
        g_cqu[:ne] += g_pg * 0.5 * c2 * exs * pg1
        g_ex = g_pg * cqu * 0.5 * c2 * pg1
        np.add.at(g_exner, e1, g_ex)
        np.add.at(g_exner, e2, g_ex)
        g_d = g_pg * cqu * 0.5 * c2 * exs / den
        np.add.at(g_rtpp, e2, g_d * inv_dc)
        np.add.at(g_rtpp, e1, -g_d * inv_dc)
    else:
        g_tend_ru[:ne] += dts * g_ru_p_new
    for x in (g_rpp, g_rtpp, g_exner, g_rho_zz):
        x[nc] = 0.0
    out.update({"rho_pp": g_rpp, "rtheta_pp": g_rtpp, "rw_p": g_rw_p, "wwAvg": g_wwavg, "ru_p": g_ru_p,
                "ruAvg": g_ruavg, "tend_ru": g_tend_ru, "tend_rho": g_tend_rho, "tend_rt": g_tend_rt,
                "tend_rw": g_tend_rw, "exner": g_exner, "theta_m": g_th, "rho_zz": g_rho_zz, "w": g_w,
                "rw": g_rw, "rw_save": g_rw_save, "cqu": g_cqu,
                PRE + "coftz_active": g_coftz, PRE + "cofwz_active": g_cofwz, PRE + "cofwt_active": g_cofwt,
                PRE + "a_tri_active": ga, PRE + "alpha_tri_active": gal, PRE + "gamma_tri_active": gg})
    return out


def divdamp_vjp(a, g):
    nc, ne = _i(a, "nCells"), _i(a, "nEdges")
    dts = _f(a, "dts")
    coef = 2.0 * _f(a, "config_smdiv") * _f(a, "config_len_disp") / dts
    coe = S.idx0(a["cellsOnEdge"][:ne], nc)
    c1, c2 = coe[:, 0], coe[:, 1]
    rt, rto, th = a["rtheta_pp"], a["rtheta_pp_old"], a["theta_m"]
    mask = (1.0 - a["specZoneMaskEdge"][:ne, None])
    d1 = -(rt[c1] - rto[c1])
    d2 = -(rt[c2] - rto[c2])
    ssum = th[c1] + th[c2]
    gr = _g(g, "ru_p", a["ru_p"])
    out = {"ru_p": gr.copy()}
    ge = gr[:ne]
    g_d2 = ge * coef * mask / ssum
    g_s = -ge * coef * (d2 - d1) * mask / (ssum * ssum)
    g_rt = np.zeros_like(rt, dtype=np.float64)
    g_rto = np.zeros_like(rto, dtype=np.float64)
    g_th = np.zeros_like(th, dtype=np.float64)
    np.add.at(g_rt, c2, -g_d2)
    np.add.at(g_rto, c2, g_d2)
    np.add.at(g_rt, c1, g_d2)
    np.add.at(g_rto, c1, -g_d2)
    np.add.at(g_th, c1, g_s)
    np.add.at(g_th, c2, g_s)
    for x in (g_rt, g_rto, g_th):
        x[nc] = 0.0
    out.update({"rtheta_pp": g_rt, "rtheta_pp_old": g_rto, "theta_m": g_th})
    return out


def smlstep_vjp(a, g):
    nc, ne, nl = _i(a, "nCells"), _i(a, "nEdges"), _i(a, "nVertLevels")
    fzm, fzp = a["fzm"][:nl], a["fzp"][:nl]
    gw = _g(g, "w_tend", a["w_tend"])
    zz = a["zz"][:nc, :nl]
    zz_i = fzm[1:] * zz[:, 1:] + fzp[1:] * zz[:, :-1]
    g_acc = gw[:nc, 1:nl] * zz_i
    out_w = gw.copy()
    out_w[:nc, 1:nl] = g_acc
    g_ut = np.zeros_like(a["u_tend"], dtype=np.float64)
    ut = a["u_tend"]
    eoc = S.idx0(a["edgesOnCell"][:nc], ne)
    n_eoc = np.asarray(a["nEdgesOnCell"][:nc]).astype(np.int64)
    sign = a["edgesOnCell_sign"][:nc]
    zb, zb3 = a["zb_cell"], a["zb3_cell"]
    for j in range(eoc.shape[1]):
        valid = (j < n_eoc) & (eoc[:, j] < ne)
        e = np.where(valid, eoc[:, j], 0)
        coef = zb[:nc, j, 1:nl] + _sgn(ut[e, 1:nl]) * zb3[:nc, j, 1:nl]
        g_ui = np.where(valid[:, None], -g_acc * coef * sign[:, j, None], 0.0)
        np.add.at(g_ut, (e, slice(1, nl)), fzm[1:] * g_ui)
        np.add.at(g_ut, (e, slice(0, nl - 1)), fzp[1:] * g_ui)
    g_ut[ne] = 0.0
    return {"w_tend": out_w, "u_tend": g_ut}


# --------------------------------------------------------------------------------------
# large-step recovery (recover_large_step.py:1090)
# --------------------------------------------------------------------------------------

def recover_vjp(a, g):
    nc, ne, nl = _i(a, "nCells"), _i(a, "nEdges"), _i(a, "nVertLevels")
    rk, ns = _i(a, "rk_step"), _i(a, "ns")
    dt = _f(a, "dt")
    inv_ns = 1.0 / float(ns)
    fzm, fzp = a["fzm"][:nl], a["fzp"][:nl]
    Sl = lambda k: a[k][:nc, :nl]
    fw = S.recover_large_step(a)
    rho_zz = fw["rho_zz"][:nc]
    rtheta_p = fw["rtheta_p"][:nc]
    theta_m = fw["theta_m"][:nc]
    rtb = Sl("rtheta_base")
    zz = Sl("zz")
    coe = S.idx0(a["cellsOnEdge"][:ne], nc)
    rz_pad = np.concatenate([rho_zz, np.ones((1, nl))])
    ru = fw["ru"][:ne]
    den_u = rz_pad[coe[:, 0]] + rz_pad[coe[:, 1]]
    zz_i = fzm[1:] * zz[:, 1:] + fzp[1:] * zz[:, :-1]
    rho_i = fzm[1:] * rho_zz[:, 1:] + fzp[1:] * rho_zz[:, :-1]
    w = fw["w"][:nc]
    gget = lambda k, like: _g(g, k, like)
    g_rho_zz = gget("rho_zz", a["rho_base"])[:nc].copy()
    g_rtp = gget("rtheta_p", a["rtheta_p_save"])[:nc].copy()
    g_rho_p = gget("rho_p", a["rho_p_save"])[:nc].copy()
    g_th = gget("theta_m", a["rtheta_p_save"])[:nc]
    out = {k: np.zeros_like(a[k], dtype=np.float64) for k in
           ("rho_p_save", "rho_pp", "rtheta_p_save", "rtheta_pp", "rw_save", "rw_p", "wwAvg", "ru_save",
            "ru_p", "ruAvg")}
    # w: interior levels (omega-derived part plus the slope fluxes of the new ru over the
    # interface density), the surface (slope fluxes of the cf-weighted ru over the
    # cf-weighted density; zero over flat terrain), the top (zero)
    gw = gget("w", a["rw_save"])[:nc]
    g_wmid = gw[:, 1:nl] / rho_i
    g_rho_i = -gw[:, 1:nl] * w[:, 1:nl] / rho_i
    g_rho_zz[:, 1:] += fzm[1:] * g_rho_i
    g_rho_zz[:, :-1] += fzp[1:] * g_rho_i
    g_rwmid = g_wmid / zz_i
    cf1, cf2, cf3 = _f(a, "cf1"), _f(a, "cf2"), _f(a, "cf3")
    den0 = cf1 * rho_zz[:, 0] + cf2 * rho_zz[:, 1] + cf3 * rho_zz[:, 2]
    g_surf = gw[:, 0] / den0
    g_den0 = -g_surf * w[:, 0]
    for q, cf in enumerate((cf1, cf2, cf3)):
        g_rho_zz[:, q] += cf * g_den0
    g_ru_slope = np.zeros((ne + 1, nl))
    eoc = S.idx0(a["edgesOnCell"][:nc], ne)
    n_eoc = np.asarray(a["nEdgesOnCell"][:nc]).astype(np.int64)
    sign = a["edgesOnCell_sign"][:nc]
    zb, zb3 = a["zb_cell"], a["zb3_cell"]
    ru_pad = np.concatenate([ru, np.zeros((1, nl))])
    for j in range(eoc.shape[1]):
        valid = (j < n_eoc) & (eoc[:, j] < ne)
        e = np.where(valid, eoc[:, j], ne)
        rs = ru_pad[e]
        fs = cf1 * rs[:, 0] + cf2 * rs[:, 1] + cf3 * rs[:, 2]
        cs = zb[:nc, j, 0] + _sgn(fs) * zb3[:nc, j, 0]
        g_fs = np.where(valid, g_surf * sign[:, j] * cs, 0.0)
        for q, cf in enumerate((cf1, cf2, cf3)):
            np.add.at(g_ru_slope, (e, q), cf * g_fs)
        fi = fzm[1:] * rs[:, 1:nl] + fzp[1:] * rs[:, :nl - 1]
        ci = zb[:nc, j, 1:nl] + _sgn(fi) * zb3[:nc, j, 1:nl]
        g_fi = np.where(valid[:, None], g_wmid * sign[:, j, None] * ci, 0.0)
        np.add.at(g_ru_slope, (e, slice(1, nl)), fzm[1:] * g_fi)
        np.add.at(g_ru_slope, (e, slice(0, nl - 1)), fzp[1:] * g_fi)
    # rw: interior levels recovered; its bottom and top levels are zero (no derivative)
    grw = gget("rw", a["rw_save"])[:nc]
    g_rwmid = g_rwmid + grw[:, 1:nl]
    out["rw_save"][:nc, 1:nl] += g_rwmid
    out["rw_p"][:nc, 1:nl] += g_rwmid
    gww = gget("wwAvg", a["wwAvg"])[:nc]
    out["rw_save"][:nc, 1:nl] += gww[:, 1:nl]
    out["wwAvg"][:nc, 1:nl] += gww[:, 1:nl] * inv_ns
    out["wwAvg"][:nc, 0] += gww[:, 0]
    out["wwAvg"][:nc, nl] += gww[:, nl]
    # edges
    gu = gget("u", a["ru_save"])[:ne]
    g_ru = gget("ru", a["ru_save"])[:ne] + gu * 2.0 / den_u + g_ru_slope[:ne]
    g_den = -gu * 2.0 * ru / (den_u * den_u)
    gz = np.zeros((nc + 1, nl))
    np.add.at(gz, coe[:, 0], g_den)
    np.add.at(gz, coe[:, 1], g_den)
    g_rho_zz += gz[:nc]
    out["ru_save"][:ne] += g_ru
    out["ru_p"][:ne] += g_ru
    gra = gget("ruAvg", a["ruAvg"])[:ne]
    out["ru_save"][:ne] += gra
    out["ruAvg"][:ne] += gra * inv_ns
    # Exner function and pressure perturbation (rk 3)
    if rk == 3:
        rcv = RGAS / (CP - RGAS)
        ex = fw["exner"][:nc]
        gp = gget("pressure_p", a["rtheta_p_save"])[:nc]
        gex = gget("exner", a["rtheta_p_save"])[:nc] + gp * zz * RGAS * (rtheta_p + rtb)
        g_rtp += gp * zz * RGAS * ex
        E = zz * (RGAS / P0) * (rtheta_p + rtb)
        g_rtp += gex * rcv * ex / E * zz * (RGAS / P0)
    # theta_m
    g_rtp += g_th / rho_zz
    g_rho_zz += -g_th * theta_m / rho_zz
    if rk == 3:
        g_rho_zz += -g_rtp * dt * Sl("rt_diabatic_tend")
    out["rtheta_p_save"][:nc] += g_rtp
    out["rtheta_pp"][:nc] += g_rtp
    g_rho_p += g_rho_zz
    out["rho_p_save"][:nc] += g_rho_p
    out["rho_pp"][:nc] += g_rho_p
    return out


# --------------------------------------------------------------------------------------
# diagnostics (solve_diagnostics.py:1052)
# --------------------------------------------------------------------------------------

def diag_vjp(a, g):
    nc, ne, nv, nl = _i(a, "nCells"), _i(a, "nEdges"), _i(a, "nVertices"), _i(a, "nVertLevels")
    rk = _i(a, "rk_step")
    dt, apvm = _f(a, "dt"), _f(a, "config_apvm_upwinding")
    u = a["u"]
    coe = S.idx0(a["cellsOnEdge"][:ne], nc)
    voe = S.idx0(a["verticesOnEdge"][:ne], nv)
    dc, dv = a["dcEdge"], a["dvEdge"]
    eov = S.idx0(a["edgesOnVertex"][:nv], ne)
    eov_sign = a["edgesOnVertex_sign"][:nv]
    eoc = S.idx0(a["edgesOnCell"][:nc], ne)
    n_eoc = np.asarray(a["nEdgesOnCell"][:nc]).astype(np.int64)
    sign = a["edgesOnCell_sign"][:nc]
    inv_area = a["invAreaCell"][:nc, None]
    iat = a["invAreaTriangle"][:nv, None]
    fw = S.solve_diagnostics(a)
    vort = fw["vorticity"][:nv]
    pvv = a["fVertex"][:nv, None] + vort
    v = fw["v"][:ne]
    ke_fact = 1.0 - 0.375
    voc = S.idx0(a["verticesOnCell"][:nc], nv)
    kite = np.asarray(a["kiteForCell"][:nc]).astype(np.int64)
    kites = a["kiteAreasOnVertex"]
    nkite = kites.shape[1]
    cv_slots = []
    for j in range(voc.shape[1]):
        valid = (j < n_eoc) & (voc[:, j] < nv) & (kite[:, j] >= 1) & (kite[:, j] <= nkite)
        vv = np.where(valid, voc[:, j], 0)
        kk = np.where(valid, kite[:, j] - 1, 0)
        cv_slots.append((valid, vv, np.where(valid, kites[vv, kk], 0.0)))
    gu = np.zeros((ne + 1, nl))
    g_pvv = np.zeros((nv + 1, nl))
    g_pve = _g(g, "pv_edge", u)[:ne]
    g_v = _g(g, "v", u)[:ne].copy()
    if apvm > 0.0:
        pvc = np.zeros((nc, nl))
        for valid, vv, wgt in cv_slots:
            pvc = pvc + np.where(valid[:, None], wgt[:, None] * pvv[vv] * inv_area, 0.0)
        pvc_pad = np.concatenate([pvc, np.zeros((1, nl))])
        pvv_pad = np.concatenate([pvv, np.zeros((1, nl))])
        grad_pvt = (pvv_pad[voe[:, 1]] - pvv_pad[voe[:, 0]]) * a["invDvEdge"][:ne, None]
        grad_pvn = (pvc_pad[coe[:, 1]] - pvc_pad[coe[:, 0]]) * a["invDcEdge"][:ne, None]
        g_delta = -g_pve * (apvm * dt)
        g_v += g_delta * grad_pvt
        gu[:ne] += g_delta * grad_pvn
        g_gt = g_delta * v * a["invDvEdge"][:ne, None]
        g_gn = g_delta * u[:ne] * a["invDcEdge"][:ne, None]
        np.add.at(g_pvv, voe[:, 1], g_gt)
        np.add.at(g_pvv, voe[:, 0], -g_gt)
        g_pvc = np.zeros((nc + 1, nl))
        np.add.at(g_pvc, coe[:, 1], g_gn)
        np.add.at(g_pvc, coe[:, 0], -g_gn)
        for valid, vv, wgt in cv_slots:
            np.add.at(g_pvv, vv, np.where(valid[:, None], g_pvc[:nc] * wgt[:, None] * inv_area, 0.0))
    out = {}
    if rk == 3:
        eoe = S.idx0(a["edgesOnEdge"][:ne], ne)
        n_eoe = np.asarray(a["nEdgesOnEdge"][:ne]).astype(np.int64)
        woe = a["weightsOnEdge"][:ne]
        for j in range(eoe.shape[1]):
            valid = (j < n_eoe) & (eoe[:, j] < ne)
            e = np.where(valid, eoe[:, j], ne)
            np.add.at(gu, e, np.where(valid, woe[:, j], 0.0)[:, None] * g_v)
    else:
        gvin = np.zeros_like(a["v_in"], dtype=np.float64)
        gvin[:ne] = g_v
        out["v_in"] = gvin
    np.add.at(g_pvv, voe[:, 0], 0.5 * g_pve)
    np.add.at(g_pvv, voe[:, 1], 0.5 * g_pve)
    g_vort = g_pvv[:nv] + _g(g, "vorticity", a["fVertex"])[:nv] if "vorticity" in g else g_pvv[:nv].copy()
    g_ke = _g(g, "ke", a["h"])[:nc]
    g_kev = np.zeros((nv + 1, nl))
    for valid, vv, wgt in cv_slots:
        np.add.at(g_kev, vv, np.where(valid[:, None], g_ke * ((1.0 - ke_fact) * wgt[:, None]) * inv_area, 0.0))
    g_kee = np.zeros((ne + 1, nl))
    g_div = _g(g, "divergence", a["h"])[:nc]
    for j in range(eoc.shape[1]):
        valid = (j < n_eoc) & (eoc[:, j] < ne)
        e = np.where(valid, eoc[:, j], ne)
        np.add.at(g_kee, e, np.where(valid[:, None], g_ke * ke_fact * 0.25 * inv_area, 0.0))
        np.add.at(gu, e, np.where(valid[:, None], g_div * inv_area * (sign[:, j] * dv[e])[:, None], 0.0))
    for j in range(eov.shape[1]):
        valid = eov[:, j] < ne
        e = np.where(valid, eov[:, j], ne)
        np.add.at(g_kee, e, np.where(valid[:, None], g_kev[:nv] * 0.25 * iat, 0.0))
        np.add.at(gu, e, np.where(valid[:, None], g_vort * iat * (eov_sign[:, j] * dc[e])[:, None], 0.0))
    gu[:ne] += g_kee[:ne] * (dc[:ne] * dv[:ne])[:, None] * 2.0 * u[:ne]
    gu[ne] = 0.0
    gh = np.zeros_like(a["h"], dtype=np.float64)
    g_he = _g(g, "h_edge", u)[:ne]
    np.add.at(gh, coe[:, 0], 0.5 * g_he)
    np.add.at(gh, coe[:, 1], 0.5 * g_he)
    gh[nc] = 0.0
    out.update({"u": gu, "h": gh})
    return out


# --------------------------------------------------------------------------------------
# large-step tendencies (dyn_tend.py:10836; sections as in stages.dyn_tend)
# --------------------------------------------------------------------------------------

def _pad_rows(a, keys, counts):
    """Inputs given with active rows only get a zero padding row (the reference hands the
    diagnostics to the later RK stages compact); returns the padded mapping and the
    original row count of every padded key."""
    a = dict(a)
    trimmed = {}
    for k in keys:
        v = a.get(k)
        if isinstance(v, np.ndarray) and v.shape[0] in counts:
            a[k] = np.concatenate([v, np.zeros((1,) + v.shape[1:], dtype=v.dtype)])
            trimmed[k] = v.shape[0]
    return a, trimmed


def dyn_tend_vjp(a, g):
    """Cotangents of the tendency stage's inputs from those of its outputs (tend_u,
    tend_w, tend_theta, tend_rho, the Euler tendencies, h_divergence, kdiff, rthdynten)."""
    nc, ne, nv, nl = _i(a, "nCells"), _i(a, "nEdges"), _i(a, "nVertices"), _i(a, "nVertLevels")
    a, trimmed = _pad_rows(a, ("u", "v", "w", "ru", "rw", "ru_save", "rw_save", "theta_m", "theta_m_save",
                               "rho_zz", "rho_edge", "divergence", "vorticity", "ke", "pv_edge", "pp",
                               "rr_save", "rt_diabatic_tend", "kdiff_in", "tend_rho_in", "tend_u_euler_in",
                               "tend_w_euler_in", "tend_theta_euler_in"),
                           (nc, ne, nv))
    rk = _i(a, "rk_step")
    dt = _f(a, "dt")
    coef3 = _f(a, "coef_3rd_order")
    c_s = _f(a, "c_s")
    len_disp = _f(a, "config_len_disp")
    del4u_div = _f(a, "config_del4u_div_factor")
    inv_dt = 1.0 / dt
    mixing = str(a["config_horiz_mixing"])
    if mixing == "2d_smagorinsky":
        h_mom_eddy_visc4 = _f(a, "config_visc4_2dsmag") * len_disp ** 3
        h_theta_eddy_visc4 = h_mom_eddy_visc4
    else:
        h_mom_eddy_visc4 = _f(a, "config_h_mom_eddy_visc4")
        h_theta_eddy_visc4 = _f(a, "config_h_theta_eddy_visc4")
    # dry columns: the moist coefficients are held constant by this sweep, so moist
    # columns are refused rather than mis-differentiated
    if "qtot" in a and np.any(np.asarray(a["qtot"]) != 0.0):
        raise NotImplementedError("derivative in moist columns")
    # the mixing and damping options (dyn_tend.py:2730-2780, 2956-2990, 3434-3456,
    # 4636-4648, 5064-5100), differentiated with the forward's branches
    v_mom = _f(a, "config_v_mom_eddy_visc2") if "config_v_mom_eddy_visc2" in a else 0.0
    v_th = _f(a, "config_v_theta_eddy_visc2") if "config_v_theta_eddy_visc2" in a else 0.0
    cam = _f(a, "config_mpas_cam_coef") if "config_mpas_cam_coef" in a else 0.0
    ncam = _i(a, "config_number_cam_damping_levels") if "config_number_cam_damping_levels" in a else 0
    mix_full = bool(a.get("config_mix_full", True))
    ray = bool(a.get("config_rayleigh_damp_u", False))
    fw = S.dyn_tend(a)
    coe = S.idx0(a["cellsOnEdge"][:ne], nc)
    e1, e2 = coe[:, 0], coe[:, 1]
    voe = S.idx0(a["verticesOnEdge"][:ne], nv)
    v1, v2 = voe[:, 0], voe[:, 1]
    eoc = S.idx0(a["edgesOnCell"][:nc], ne)
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
    th = a["theta_m"]
    zz = a["zz"]
    pp = a["pp"]
    qtot = a["qtot"]
    rho_zz = a["rho_zz"]
    rtd = a["rt_diabatic_tend"]

    def slots():
        for j in range(eoc.shape[1]):
            valid = (j < n_eoc) & (eoc[:, j] < ne)
            yield j, valid, np.where(valid, eoc[:, j], 0)

    G = {k: _g(g, k, fw[k]) for k in ("tend_u", "tend_w", "tend_theta", "tend_rho", "tend_u_euler",
                                       "tend_w_euler", "tend_theta_euler", "h_divergence", "kdiff",
                                       "rthdynten")}
    Z = lambda x: np.zeros_like(x, dtype=np.float64)
    gu, gv, gw, gru, grw = Z(u), Z(v), Z(w), Z(ru), Z(rw)
    gru_save, grw_save = Z(a["ru_save"]), Z(a["rw_save"])
    gth, gths = Z(th), Z(a["theta_m_save"])
    grho_edge, grho_zz = Z(rho_edge), Z(rho_zz)
    gdiv, gvort, gke, gpv = Z(a["divergence"]), Z(a["vorticity"]), Z(a["ke"]), Z(a["pv_edge"])
    gpp, grr_save, grtd = Z(pp), Z(a["rr_save"]), Z(rtd)
    gkd = np.zeros((nc + 1, nl))
    ghd = np.zeros((nc + 1, nl))
    gdpdz = np.zeros((nc + 1, nl))
    out = {}

    kdiff = fw["kdiff"]
    tend_rho = fw["tend_rho"]
    ia = inv_area[:nc, None]
    adv = S.idx0(a["advCellsForEdge"][:ne], nc)
    n_adv = np.asarray(a["nAdvCellsForEdge"][:ne]).astype(np.int64)
    acoef, acoef3 = a["adv_coefs"][:ne], a["adv_coefs_3rd"][:ne]
    dpdz = np.zeros((nc + 1, nl))
    dpdz[:nc] = -GRAVITY * (a["rb"][:nc] * qtot[:nc] + a["rr_save"][:nc] * (1.0 + qtot[:nc]))

    # ================= theta tendency
    g_ttfull = G["tend_theta"][:nc]
    grho_zz[:nc] += g_ttfull * rtd[:nc]
    grtd[:nc] += g_ttfull * rho_zz[:nc]
    g_tte = g_ttfull + G["tend_theta_euler"][:nc]
    g_rth = G["rthdynten"][:nc]
    rthd = fw["rthdynten"][:nc]
    g_tt2 = g_ttfull + g_rth / rho_zz[:nc]
    g_trho = G["tend_rho"][:nc] - g_rth * th[:nc] / rho_zz[:nc]
    gth[:nc] += -g_rth * tend_rho[:nc] / rho_zz[:nc]
    grho_zz[:nc] += -g_rth * rthd / rho_zz[:nc]
    g_tt1 = g_tt2 * ia
    g_wdtz = np.zeros((nc, nl + 1))
    g_wdtz[:, 1:] += -g_tt2 * rdzw[None, :]
    g_wdtz[:, :nl] += g_tt2 * rdzw[None, :]
    thc, thsc, rwc, rwsc = th[:nc], a["theta_m_save"][:nc], rw[:nc], a["rw_save"][:nc]
    gthc, gthsc, grwc, grwsc = gth[:nc], gths[:nc], grw[:nc], grw_save[:nc]
    for k in range(1, nl):
        gwd = g_wdtz[:, k]
        fm, fp = fzm[k], fzp[k]
        if k == nl - 1 and k != 1:
            grwsc[:, k] += gwd * (fm * thc[:, k] + fp * thc[:, k - 1])
            gthc[:, k] += gwd * rwsc[:, k] * fm
            gthc[:, k - 1] += gwd * rwsc[:, k] * fp
            continue
        if k == 1:
            grwc[:, k] += gwd * (fm * thc[:, k] + fp * thc[:, k - 1])
            gthc[:, k] += gwd * rwc[:, k] * fm
            gthc[:, k - 1] += gwd * rwc[:, k] * fp
        else:
            d = flux3_grads(thc[:, k - 2], thc[:, k - 1], thc[:, k], thc[:, k + 1], rwc[:, k], coef3)
            gthc[:, k - 2] += gwd * d[0]
            gthc[:, k - 1] += gwd * d[1]
            gthc[:, k] += gwd * d[2]
            gthc[:, k + 1] += gwd * d[3]
            grwc[:, k] += gwd * d[4]
        tse = fm * thsc[:, k] + fp * thsc[:, k - 1]
        grwsc[:, k] += gwd * tse
        grwc[:, k] -= gwd * tse
        gthsc[:, k] += gwd * (rwsc[:, k] - rwc[:, k]) * fm
        gthsc[:, k - 1] += gwd * (rwsc[:, k] - rwc[:, k]) * fp
    # horizontal advection of theta: edge fluxes ru * sum_m cf_m theta[adv_m]
    g_fte = np.zeros((ne + 1, nl))
    for j, valid, e in slots():
        np.add.at(g_fte, e, np.where(valid[:, None], -g_tt1 * sign[:, j, None], 0.0))
    if rk > 1:
        ths = a["theta_m_save"]
        for j, valid, e in slots():
            wj = np.where(valid, sign[:, j] * dv[e], 0.0)[:, None]
            the = 0.5 * (ths[e2[e]] + ths[e1[e]])
            gx = -g_tt1
            np.add.at(gru_save, e, np.where(valid[:, None], gx * wj * the, 0.0))
            np.add.at(gru, e, np.where(valid[:, None], -gx * wj * the, 0.0))
            gthe = np.where(valid[:, None], gx * wj * (a["ru_save"][e] - ru[e]), 0.0)
            np.add.at(gths, e2[e], 0.5 * gthe)
            np.add.at(gths, e1[e], 0.5 * gthe)
    flt = np.zeros((ne, nl))
    sg_ru = _sgn(ru[:ne])
    for m in range(adv.shape[1]):
        vm = m < n_adv
        cell = np.where(vm, adv[:, m], nc)
        cf = (acoef[:, m][:, None] + sg_ru * acoef3[:, m][:, None]) * vm[:, None]
        flt = flt + cf * th[cell]
    gru[:ne] += g_fte[:ne] * flt
    gflt = g_fte[:ne] * ru[:ne]
    for m in range(adv.shape[1]):
        vm = m < n_adv
        cell = np.where(vm, adv[:, m], nc)
        cf = (acoef[:, m][:, None] + sg_ru * acoef3[:, m][:, None]) * vm[:, None]
        np.add.at(gth, cell, gflt * cf)
    # theta mixing (rk 1)
    if rk == 1:
        g_dst = np.zeros((nc + 1, nl))
        if h_theta_eddy_visc4 > 0.0:
            for j, valid, e in slots():
                es = np.where(valid, a["meshScalingDel4"][e] * (h_theta_eddy_visc4 * 1.0 * inv_area[:nc]) * dv[e]
                              * sign[:, j] * inv_dc[e], 0.0)[:, None]
                np.add.at(g_dst, e2[e], -g_tte * es)
                np.add.at(g_dst, e1[e], g_tte * es)
        for j, valid, e in slots():
            es = np.where(valid, inv_area[:nc] * sign[:, j] * dv[e] * inv_dc[e], 0.0)[:, None]
            pr = a["meshScalingDel2"][e][:, None]
            c1, c2 = e1[e], e2[e]
            dth = th[c2] - th[c1]
            flux = es * dth * rho_edge[e]
            kd = 0.5 * (kdiff[c1] + kdiff[c2])
            g_flux = g_tte * kd * pr + g_dst[:nc]
            g_kdm = g_tte * flux * 0.5 * pr
            np.add.at(gkd, c1, g_kdm)
            np.add.at(gkd, c2, g_kdm)
            np.add.at(gth, c2, g_flux * es * rho_edge[e])
            np.add.at(gth, c1, -g_flux * es * rho_edge[e])
            np.add.at(grho_edge, e, g_flux * es * dth)
        if v_th > 0.0 and nl > 2:  # vertical mixing of theta
            zg = a["zgrid"][:nc]
            z1, z2, z3, z4 = zg[:, 0:nl - 2], zg[:, 1:nl - 1], zg[:, 2:nl], zg[:, 3:nl + 1]
            zm, z0, zp = 0.5 * (z1 + z2), 0.5 * (z2 + z3), 0.5 * (z3 + z4)
            thv = th[:nc] if mix_full else th[:nc] - a["t_init"][:nc]
            diff = (thv[:, 2:nl] - thv[:, 1:nl - 1]) / (zp - z0) - (thv[:, 1:nl - 1] - thv[:, :nl - 2]) / (z0 - zm)
            den = 0.5 * (zp - zm)
            gt = g_tte[:, 1:nl - 1]
            grho_zz[:nc, 1:nl - 1] += gt * v_th * diff / den
            av = gt * v_th * rho_zz[:nc, 1:nl - 1] / den
            gth[:nc, 2:nl] += av / (zp - z0)
            gth[:nc, 1:nl - 1] += -av / (zp - z0) - av / (z0 - zm)
            gth[:nc, :nl - 2] += av / (z0 - zm)
    else:
        out["tend_theta_euler_in"] = np.concatenate([g_tte, np.zeros((1, nl))])

    # ================= w tendency
    g_tw = G["tend_w"][:nc]
    g_twe = g_tw + G["tend_w_euler"][:nc]
    g_tw2 = g_tw
    g_tw1 = np.zeros((nc, nl + 1))
    g_tw1[:, 1:nl] = g_tw2[:, 1:nl] * ia
    g_wdwz = np.zeros((nc, nl + 2))
    g_wdwz[:, 2:nl + 1] += -g_tw2[:, 1:nl] * rdzu[None, 1:]
    g_wdwz[:, 1:nl] += g_tw2[:, 1:nl] * rdzu[None, 1:]
    wc = w[:nc]
    gwc = gw[:nc]
    for k in range(1, nl):
        gwd = g_wdwz[:, k]
        if k == 1 or k == nl - 1:
            grwc[:, k] += gwd * 0.25 * (wc[:, k] + wc[:, k - 1])
            grwc[:, k - 1] += gwd * 0.25 * (wc[:, k] + wc[:, k - 1])
            gwc[:, k] += gwd * 0.25 * (rwc[:, k] + rwc[:, k - 1])
            gwc[:, k - 1] += gwd * 0.25 * (rwc[:, k] + rwc[:, k - 1])
        else:
            ua = 0.5 * (rwc[:, k] + rwc[:, k - 1])
            d = flux3_grads(wc[:, k - 2], wc[:, k - 1], wc[:, k], wc[:, k + 1], ua, 1.0)
            gwc[:, k - 2] += gwd * d[0]
            gwc[:, k - 1] += gwd * d[1]
            gwc[:, k] += gwd * d[2]
            gwc[:, k + 1] += gwd * d[3]
            grwc[:, k] += 0.5 * gwd * d[4]
            grwc[:, k - 1] += 0.5 * gwd * d[4]
    # horizontal advection of w: edge fluxes ru_w * sum_m cf_m w[adv_m]
    g_fwe = np.zeros((ne + 1, nl))
    for j, valid, e in slots():
        np.add.at(g_fwe, (e, slice(1, nl)), np.where(valid[:, None], -g_tw1[:, 1:nl] * sign[:, j, None], 0.0))
    ru_w = np.zeros((ne, nl))
    ru_w[:, 1:] = fzm[1:] * ru[:ne, 1:nl] + fzp[1:] * ru[:ne, :nl - 1]
    sg_w = _sgn(ru_w)
    flw = np.zeros((ne, nl))
    for m in range(adv.shape[1]):
        vm = m < n_adv
        cell = np.where(vm, adv[:, m], nc)
        cf = (acoef[:, m][:, None] + sg_w * acoef3[:, m][:, None]) * vm[:, None]
        flw[:, 1:] = flw[:, 1:] + cf[:, 1:] * w[cell, 1:nl]
    g_ruw = g_fwe[:ne] * flw
    gru[:ne, 1:nl] += g_ruw[:, 1:] * fzm[1:]
    gru[:ne, :nl - 1] += g_ruw[:, 1:] * fzp[1:]
    gflw = g_fwe[:ne] * ru_w
    for m in range(adv.shape[1]):
        vm = m < n_adv
        cell = np.where(vm, adv[:, m], nc)
        cf = (acoef[:, m][:, None] + sg_w * acoef3[:, m][:, None]) * vm[:, None]
        np.add.at(gw, (cell, slice(1, nl)), gflw[:, 1:] * cf[:, 1:])
    if rk == 1:
        cqw = a["cqw"]
        gtw_e = g_twe[:, 1:nl]
        gpp[:nc, 1:] += -gtw_e * cqw[:nc, 1:nl] * rdzu[None, 1:]
        gpp[:nc, :nl - 1] += gtw_e * cqw[:nc, 1:nl] * rdzu[None, 1:]
        gdpdz[:nc, 1:] += gtw_e * cqw[:nc, 1:nl] * fzm[None, 1:]
        gdpdz[:nc, :nl - 1] += gtw_e * cqw[:nc, 1:nl] * fzp[None, 1:]
        # w mixing
        g_dsw = np.zeros((nc + 1, nl + 1))
        if h_mom_eddy_visc4 > 0.0:
            for j, valid, e in slots():
                es = np.where(valid, a["meshScalingDel4"][e] * (h_mom_eddy_visc4 * inv_area[:nc]) * dv[e]
                              * sign[:, j] * inv_dc[e], 0.0)[:, None]
                np.add.at(g_dsw, (e2[e], slice(1, nl)), -g_twe[:, 1:nl] * es)
                np.add.at(g_dsw, (e1[e], slice(1, nl)), g_twe[:, 1:nl] * es)
        for j, valid, e in slots():
            es = np.where(valid, 0.5 * inv_area[:nc] * sign[:, j] * dv[e] * inv_dc[e], 0.0)[:, None]
            c1, c2 = e1[e], e2[e]
            rsum = rho_edge[e, 1:nl] + rho_edge[e, :nl - 1]
            dw = w[c2, 1:nl] - w[c1, 1:nl]
            flux = es * rsum * dw
            kd = 0.25 * (kdiff[c1, 1:nl] + kdiff[c2, 1:nl] + kdiff[c1, :nl - 1] + kdiff[c2, :nl - 1])
            msd = a["meshScalingDel2"][e][:, None]
            g_flux = g_twe[:, 1:nl] * msd * kd + g_dsw[:nc, 1:nl]
            g_kd4 = g_twe[:, 1:nl] * flux * msd * 0.25
            np.add.at(gkd, (c1, slice(1, nl)), g_kd4)
            np.add.at(gkd, (c2, slice(1, nl)), g_kd4)
            np.add.at(gkd, (c1, slice(0, nl - 1)), g_kd4)
            np.add.at(gkd, (c2, slice(0, nl - 1)), g_kd4)
            g_rs = g_flux * es * dw
            np.add.at(grho_edge, (e, slice(1, nl)), g_rs)
            np.add.at(grho_edge, (e, slice(0, nl - 1)), g_rs)
            np.add.at(gw, (c2, slice(1, nl)), g_flux * es * rsum)
            np.add.at(gw, (c1, slice(1, nl)), -g_flux * es * rsum)
        if v_mom > 0.0:  # vertical mixing of w
            rz = rho_zz[:nc]
            w_up = (wc[:, 2:nl + 1] - wc[:, 1:nl]) * rdzw[1:nl]
            w_down = (wc[:, 1:nl] - wc[:, :nl - 1]) * rdzw[:nl - 1]
            b = g_twe[:, 1:nl] * v_mom * rdzu[1:nl]
            grho_zz[:nc, 1:nl] += 0.5 * b * (w_up - w_down)
            grho_zz[:nc, :nl - 1] += 0.5 * b * (w_up - w_down)
            av = b * 0.5 * (rz[:, 1:nl] + rz[:, :nl - 1])
            gw[:nc, 2:nl + 1] += av * rdzw[1:nl]
            gw[:nc, 1:nl] += -av * rdzw[1:nl] - av * rdzw[:nl - 1]
            gw[:nc, :nl - 1] += av * rdzw[:nl - 1]
    else:
        gi = np.zeros((nc + 1, nl + 1))
        gi[:nc] = G["tend_w_euler"][:nc]  # passed through at every level
        gi[:nc, 1:nl] += g_tw[:, 1:nl]
        out["tend_w_euler_in"] = gi

    # ================= u tendency
    g_tu = G["tend_u"][:ne]
    g_teu = g_tu + G["tend_u_euler"][:ne]
    hdp = fw["h_divergence"]
    ke = a["ke"]
    eoe = S.idx0(a["edgesOnEdge"][:ne], ne)
    n_eoe = np.asarray(a["nEdgesOnEdge"][:ne]).astype(np.int64)
    woe = a["weightsOnEdge"][:ne]
    pv = a["pv_edge"]
    q = np.zeros((ne, nl))
    for j in range(eoe.shape[1]):
        valid = (j < n_eoe) & (eoe[:, j] < ne)
        e = np.where(valid, eoe[:, j], 0)
        q = q + np.where(valid, woe[:, j], 0.0)[:, None] * u[e] * 0.5 * (pv[:ne] + pv[e])
    dke = (ke[e2] - ke[e1]) * inv_dc[:ne, None]
    grho_edge[:ne] += g_tu * (q - dke)
    gq = g_tu * rho_edge[:ne]
    gke_e = g_tu * rho_edge[:ne] * inv_dc[:ne, None]
    np.add.at(gke, e2, -gke_e)
    np.add.at(gke, e1, gke_e)
    gu[:ne] += -g_tu * 0.5 * (hdp[e1] + hdp[e2])
    np.add.at(ghd, e1, -g_tu * u[:ne] * 0.5)
    np.add.at(ghd, e2, -g_tu * u[:ne] * 0.5)
    for j in range(eoe.shape[1]):
        valid = (j < n_eoe) & (eoe[:, j] < ne)
        e = np.where(valid, eoe[:, j], ne)
        wj = np.where(valid, woe[:, j], 0.0)[:, None]
        np.add.at(gu, e, gq * wj * 0.5 * (pv[:ne] + pv[e]))
        gpv[:ne] += gq * wj * u[e] * 0.5
        np.add.at(gpv, e, gq * wj * u[e] * 0.5)
    g_wduz = np.zeros((ne, nl + 1))
    g_wduz[:, 1:] += -g_tu * rdzw[None, :]
    g_wduz[:, :nl] += g_tu * rdzw[None, :]
    rw_e = 0.5 * (rw[e1] + rw[e2])
    g_rwe = np.zeros((ne, nl + 1))
    ue = u[:ne]
    gue = gu[:ne]
    for k in range(1, nl):
        gwd = g_wduz[:, k]
        if k == 1 or k == nl - 1:
            g_rwe[:, k] += gwd * (fzm[k] * ue[:, k] + fzp[k] * ue[:, k - 1])
            gue[:, k] += gwd * rw_e[:, k] * fzm[k]
            gue[:, k - 1] += gwd * rw_e[:, k] * fzp[k]
        else:
            d = flux3_grads(ue[:, k - 2], ue[:, k - 1], ue[:, k], ue[:, k + 1], rw_e[:, k], 1.0)
            gue[:, k - 2] += gwd * d[0]
            gue[:, k - 1] += gwd * d[1]
            gue[:, k] += gwd * d[2]
            gue[:, k + 1] += gwd * d[3]
            g_rwe[:, k] += gwd * d[4]
    np.add.at(grw, e1, 0.5 * g_rwe)
    np.add.at(grw, e2, 0.5 * g_rwe)
    if ray:  # Rayleigh damping of u: tend_u - rho_edge u damp on the top levels
        nray = _i(a, "config_number_rayleigh_damp_u_levels")
        coef = 1.0 / (float(nray) * (_f(a, "config_rayleigh_damp_u_timescale_days") * 86400.0))
        k0 = nl - nray
        damp = ((np.arange(k0, nl, dtype=np.float64) + 1.0) - float(k0)) * coef
        grho_edge[:ne, k0:] += -g_tu[:, k0:] * u[:ne, k0:] * damp[None, :]
        gu[:ne, k0:] += -g_tu[:, k0:] * rho_edge[:ne, k0:] * damp[None, :]
    if rk == 1:
        zzm = 0.5 * (zz[e2] + zz[e1])
        cqu = a["cqu"][:ne]
        gpg = -g_teu * cqu * inv_dc[:ne, None] / zzm
        np.add.at(gpp, e2, gpg)
        np.add.at(gpp, e1, -gpg)
        gdz = g_teu * cqu * 0.5 * a["zxu"][:ne]
        np.add.at(gdpdz, e1, gdz)
        np.add.at(gdpdz, e2, gdz)
        div, vort = a["divergence"], a["vorticity"]
        r_dc = inv_dc[:ne, None]
        r_dv = np.minimum(inv_dv[:ne], 4.0 * inv_dc[:ne])[:, None]
        u_diff = (div[e2] - div[e1]) * r_dc - (vort[v2] - vort[v1]) * r_dv
        kdiffu = 0.5 * (kdiff[e1] + kdiff[e2])
        msd2 = a["meshScalingDel2"][:ne, None]
        grho_edge[:ne] += g_teu * kdiffu * u_diff * msd2
        gkdu = g_teu * rho_edge[:ne] * u_diff * msd2
        np.add.at(gkd, e1, 0.5 * gkdu)
        np.add.at(gkd, e2, 0.5 * gkdu)
        g_ud = g_teu * rho_edge[:ne] * kdiffu * msd2
        if h_mom_eddy_visc4 > 0.0:
            eov = S.idx0(a["edgesOnVertex"][:nv], ne)
            eov_sign = a["edgesOnVertex_sign"][:nv]
            delsq_u = u_diff
            dsv = np.zeros((nv + 1, nl))
            for j in range(eov.shape[1]):
                valid = eov[:, j] < ne
                e = np.where(valid, eov[:, j], 0)
                es = np.where(valid, a["invAreaTriangle"][:nv] * dc[e] * eov_sign[:, j], 0.0)[:, None]
                dsv[:nv] = dsv[:nv] + es * delsq_u[e]
            dsd = np.zeros((nc + 1, nl))
            for j, valid, e in slots():
                es = np.where(valid, inv_area[:nc] * dv[e] * sign[:, j], 0.0)[:, None]
                dsd[:nc] = dsd[:nc] + es * delsq_u[e]
            u_mix = a["meshScalingDel4"][:ne] * h_mom_eddy_visc4
            r_dc4 = (u_mix * del4u_div * inv_dc[:ne])[:, None]
            r_dv4 = (u_mix * np.minimum(inv_dv[:ne], 4.0 * inv_dc[:ne]))[:, None]
            u_diff4 = (dsd[e2] - dsd[e1]) * r_dc4 - (dsv[v2] - dsv[v1]) * r_dv4
            grho_edge[:ne] += -g_teu * u_diff4
            gud4 = -g_teu * rho_edge[:ne]
            gdsd = np.zeros((nc + 1, nl))
            gdsv = np.zeros((nv + 1, nl))
            np.add.at(gdsd, e2, gud4 * r_dc4)
            np.add.at(gdsd, e1, -gud4 * r_dc4)
            np.add.at(gdsv, v2, -gud4 * r_dv4)
            np.add.at(gdsv, v1, gud4 * r_dv4)
            gdel = np.zeros((ne + 1, nl))
            for j in range(eov.shape[1]):
                valid = eov[:, j] < ne
                e = np.where(valid, eov[:, j], ne)
                es = np.where(valid, a["invAreaTriangle"][:nv] * dc[e] * eov_sign[:, j], 0.0)[:, None]
                np.add.at(gdel, e, gdsv[:nv] * es)
            for j, valid, e in slots():
                e_ = np.where(valid, e, ne)
                es = np.where(valid, inv_area[:nc] * dv[e] * sign[:, j], 0.0)[:, None]
                np.add.at(gdel, e_, gdsd[:nc] * es)
            g_ud = g_ud + gdel[:ne]
        if v_mom > 0.0 and nl > 2:  # vertical mixing of u
            zg = a["zgrid"]
            zi = lambda k0, k1: 0.5 * (zg[e1, k0:k1] + zg[e2, k0:k1])
            z1, z2, z3, z4 = zi(0, nl - 2), zi(1, nl - 1), zi(2, nl), zi(3, nl + 1)
            zm, z0, zp = 0.5 * (z1 + z2), 0.5 * (z2 + z3), 0.5 * (z3 + z4)
            uu = u[:ne]
            if not mix_full:
                ang = a["angleEdge"][:ne, None]
                uu = uu - a["u_init"][None, :nl] * np.cos(ang) - a["v_init"][None, :nl] * np.sin(ang)
            sdiff = (uu[:, 2:nl] - uu[:, 1:nl - 1]) / (zp - z0) - (uu[:, 1:nl - 1] - uu[:, :nl - 2]) / (z0 - zm)
            den = 0.5 * (zp - zm)
            gt = g_teu[:, 1:nl - 1]
            grho_edge[:ne, 1:nl - 1] += gt * v_mom * sdiff / den
            av = gt * rho_edge[:ne, 1:nl - 1] * v_mom / den
            gu[:ne, 2:nl] += av / (zp - z0)
            gu[:ne, 1:nl - 1] += -av / (zp - z0) - av / (z0 - zm)
            gu[:ne, :nl - 2] += av / (z0 - zm)
        np.add.at(gdiv, e2, g_ud * r_dc)
        np.add.at(gdiv, e1, -g_ud * r_dc)
        np.add.at(gvort, v2, -g_ud * r_dv)
        np.add.at(gvort, v1, g_ud * r_dv)
    else:
        gi = np.zeros((ne + 1, nl))
        gi[:ne] = g_teu
        out["tend_u_euler_in"] = gi

    # ================= kdiff
    gkd_out = G["kdiff"][:nc] + gkd[:nc]
    if rk == 1:
        if mixing == "2d_smagorinsky":
            d_diag = np.zeros((nc, nl))
            d_off = np.zeros((nc, nl))
            for j, valid, e in slots():
                ca = a["defc_a"][:nc, j][:, None]
                cb = a["defc_b"][:nc, j][:, None]
                d_diag = np.where(valid[:, None], (d_diag + ca * u[e]) - cb * v[e], d_diag)
                d_off = np.where(valid[:, None], (d_off + cb * u[e]) + ca * v[e], d_off)
            s2 = d_diag ** 2 + d_off ** 2
            sq = np.sqrt(s2)
            A_ = (c_s * len_disp) ** 2 * sq
            cap = (0.01 * len_disp ** 2) * inv_dt
            if cam > 0.0 and ncam > 0:  # max(kdiff, CAM floor) on the top levels: the branch taken
                kd_s = np.minimum(A_, cap)
                base = 4.0 * 2.0833 * len_disp * cam
                gkd_out = gkd_out.copy()
                for k in range(nl - ncam, nl):
                    fl = base * (1.0 - float(nl - (k + 1)) / float(ncam))
                    gkd_out[:, k] *= np.where(kd_s[:, k] > fl, 1.0, np.where(kd_s[:, k] == fl, 0.5, 0.0))
            gA = np.where(A_ < cap, gkd_out, np.where(A_ == cap, 0.5 * gkd_out, 0.0))
            gs = gA * (c_s * len_disp) ** 2 * 0.5 / sq
            gdd = gs * 2.0 * d_diag
            gdo = gs * 2.0 * d_off
            for j, valid, e in slots():
                ca = a["defc_a"][:nc, j][:, None]
                cb = a["defc_b"][:nc, j][:, None]
                e_ = np.where(valid, e, ne)
                vm = valid[:, None]
                np.add.at(gu, e_, np.where(vm, gdd * ca + gdo * cb, 0.0))
                np.add.at(gv, e_, np.where(vm, -gdd * cb + gdo * ca, 0.0))
    else:
        gi = np.zeros((nc + 1, nl))
        gi[:nc] = gkd_out
        out["kdiff_in"] = gi

    # ================= density tendency and the mass-flux divergence
    ghd[:nc] += G["h_divergence"][:nc]
    if rk == 1:
        ghd[:nc] += -g_trho
        grw[:nc, 1:] += -g_trho * rdzw[None, :]
        grw[:nc, :nl] += g_trho * rdzw[None, :]
    else:
        gi = np.zeros((nc + 1, nl))
        gi[:nc] = g_trho
        out["tend_rho_in"] = gi
    for j, valid, e in slots():
        e_ = np.where(valid, e, ne)
        wgt = np.where(valid, sign[:, j] * dv[e], 0.0)[:, None]
        np.add.at(gru, e_, ghd[:nc] * ia * wgt)
    grr_save[:nc] += gdpdz[:nc] * (-GRAVITY) * (1.0 + qtot[:nc])

    for x, n in ((gu, ne), (gv, ne), (gru, ne), (gru_save, ne), (grho_edge, ne), (gpv, ne),
                 (gw, nc), (grw, nc), (grw_save, nc), (gth, nc), (gths, nc), (grho_zz, nc), (gdiv, nc),
                 (gke, nc), (gpp, nc), (grr_save, nc), (grtd, nc), (gvort, nv)):
        x[n] = 0.0
    out.update({"u": gu, "v": gv, "w": gw, "ru": gru, "rw": grw, "ru_save": gru_save, "rw_save": grw_save,
                "theta_m": gth, "theta_m_save": gths, "rho_edge": grho_edge, "rho_zz": grho_zz,
                "divergence": gdiv, "vorticity": gvort, "ke": gke, "pv_edge": gpv, "pp": gpp,
                "rr_save": grr_save, "rt_diabatic_tend": grtd})
    for k, n in trimmed.items():
        if k in out:
            out[k] = out[k][:n]
    return out


# --------------------------------------------------------------------------------------
# whole large step and preparation
# --------------------------------------------------------------------------------------

# step-boundary fields that carry derivatives from one large step into the next
# (the reference's _INTER_STEP_PROGNOSTIC_KEYS | _INTER_STEP_EXACT_DIAGNOSTIC_KEYS,
# atmosphere_model.py:156-202, restricted to what the dry dynamics read)
CARRIED = ("u", "v", "w", "ru", "rw", "theta_m", "rho_zz", "rho_p", "rtheta_p", "exner", "pressure_p",
           "h_edge", "divergence", "vorticity", "ke", "pv_edge")
# (save field, the state field it copies) at the start of every dynamics substep
SAVES = (("ru_save", "ru"), ("rw_save", "rw"), ("rtheta_p_save", "rtheta_p"), ("rho_p_save", "rho_p"),
         ("theta_m_save", "theta_m"), ("rr_save", "rho_p"))
COEFS = ("cofwz_active", "coftz_active", "cofwt_active", "a_tri_active", "alpha_tri_active", "gamma_tri_active")
WORK = ("ru_p", "rw_p", "rho_pp", "rtheta_pp", "rtheta_pp_old", "ruAvg", "wwAvg")
TENDS = ("tend_u", "tend_w", "tend_theta", "tend_rho", "tend_u_euler", "tend_w_euler", "tend_theta_euler",
         "kdiff", "tend_rw")


class _Acc(dict):
    """Cotangent accumulators keyed by field name (missing = zero)."""

    def add(self, k, v):
        if v is None:
            return
        if k in self:
            self[k] = self[k] + v
        else:
            self[k] = np.array(v, dtype=np.float64, copy=True)

    def take(self, k):
        return self.pop(k, None)


def _tape(stepper, fn, *args):
    """Run a Stepper method recording every stage call's inputs (copied) in order."""
    rec = []

    def on_stage(name, a, out):
        rec.append((name, {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in a.items()}))

    old = stepper.on_stage
    stepper.on_stage = on_stage
    try:
        result = fn(*args)
    finally:
        stepper.on_stage = old
    return result, rec


def _route_out(acc, mapping):
    """Output cotangents of a stage (stage output name -> accumulator name); the
    accumulators of the overwritten fields are cleared."""
    g = {}
    for out_name, var in mapping.items():
        v = acc.take(var)
        if v is not None:
            g[out_name] = v
    return g


def _route_in(acc, grads, mapping):
    for in_name, var in mapping.items():
        if in_name in grads:
            acc.add(var, grads[in_name])


def step_vjp(stepper, st, dt, g_out):
    """Reverse sweep of one large step (Stepper.srk3_step) from the state ``st`` at the
    step's start: ``g_out`` holds cotangents of the step's output fields (CARRIED names);
    returns the cotangents of the step's input fields (CARRIED names).  The step is first
    recomputed from ``st`` with every stage call's inputs recorded (the reference's
    per-step checkpoint with recomputation, autodiff/checkpoint.py:106-254)."""
    from .step import STAGE_NAMES, COUPLED_STAGE_NAMES, rk_weights
    _, rec = _tape(stepper, stepper.srk3_step, st, dt)
    names = {v: k for k, v in STAGE_NAMES.items()}
    names.update({v: k for k, v in COUPLED_STAGE_NAMES.items()})
    rec = [(names[n], a) for n, a in rec]
    acc = _Acc()
    for k, v in g_out.items():
        if k in CARRIED:
            acc.add(k, v)
        elif k == "rho_edge":
            acc.add("h_edge", v)

    def pop(key):
        k, a = rec.pop()
        assert k == key, (k, key)
        return a

    split = stepper.split
    dt_dyn = dt / split
    _, _, nsub = rk_weights(dt_dyn, stepper.ns, stepper.order)
    pop("reconstruct")
    if not stepper.coupled and stepper.advect:
        while rec and rec[-1][0] in ("scalars", "scalars_mono"):
            rec.pop()
    for sub in range(split, 0, -1):
        if sub < split:  # the saves refreshed from the state after substep `sub`
            for save, src in SAVES:
                acc.add(src, acc.take(save))
        for rk in (3, 2, 1):
            a = pop("diag")
            g = _route_out(acc, {"h_edge": "h_edge", "v": "v", "divergence": "divergence",
                                 "vorticity": "vorticity", "ke": "ke", "pv_edge": "pv_edge"})
            gi = diag_vjp(a, g)
            _route_in(acc, gi, {"u": "u", "h": "rho_zz", "v_in": "v"})
            while rec and rec[-1][0] in ("scalars", "scalars_mono"):
                rec.pop()
            a = pop("recover")
            mp = {"rho_p": "rho_p", "rho_zz": "rho_zz", "rtheta_p": "rtheta_p", "theta_m": "theta_m",
                  "u": "u", "ru": "ru", "w": "w", "rw": "rw", "ruAvg": "ruAvg", "wwAvg": "wwAvg"}
            if rk == 3:
                mp.update({"exner": "exner", "pressure_p": "pressure_p"})
            gi = recover_vjp(a, _route_out(acc, mp))
            _route_in(acc, gi, {"rho_p_save": "rho_p_save", "rho_pp": "rho_pp", "rtheta_p_save": "rtheta_p_save",
                                "rtheta_pp": "rtheta_pp", "wwAvg": "wwAvg", "rw_save": "rw_save", "rw_p": "rw_p",
                                "ruAvg": "ruAvg", "ru_save": "ru_save", "ru_p": "ru_p"})
            for _small in range(nsub[rk - 1], 0, -1):
                a = pop("divdamp")
                gi = divdamp_vjp(a, _route_out(acc, {"ru_p": "ru_p"}))
                _route_in(acc, gi, {"ru_p": "ru_p", "rtheta_pp": "rtheta_pp", "rtheta_pp_old": "rtheta_pp_old",
                                    "theta_m": "theta_m_save"})
                a = pop("acoustic")
                gi = acoustic_vjp(a, _route_out(acc, {k: k for k in WORK}))
                _route_in(acc, gi, {**{k: k for k in WORK}, "tend_ru": "tend_u", "tend_rho": "tend_rho",
                                    "tend_rt": "tend_theta", "tend_rw": "tend_rw", "exner": "exner",
                                    "theta_m": "theta_m_save", "rho_zz": "rho_zz", "rw": "rw",
                                    "rw_save": "rw_save", "w": "w",
                                    **{PRE + c: c for c in COEFS}})
            a = pop("smlstep")
            gi = smlstep_vjp(a, _route_out(acc, {"w_tend": "tend_rw"}))
            _route_in(acc, gi, {"w_tend": "tend_w", "u_tend": "tend_u"})
            a = pop("dyn_tend")
            gi = dyn_tend_vjp(a, _route_out(acc, {k: k for k in TENDS if k != "tend_rw"}))
            _route_in(acc, gi, {"u": "u", "v": "v", "w": "w", "ru": "ru", "rw": "rw", "ru_save": "ru_save",
                                "rw_save": "rw_save", "theta_m": "theta_m", "theta_m_save": "theta_m_save",
                                "rho_zz": "rho_zz", "rho_edge": "h_edge", "divergence": "divergence",
                                "vorticity": "vorticity", "ke": "ke", "pv_edge": "pv_edge", "pp": "pressure_p",
                                "rr_save": "rr_save", "tend_rho_in": "tend_rho", "kdiff_in": "kdiff",
                                "tend_u_euler_in": "tend_u_euler", "tend_w_euler_in": "tend_w_euler",
                                "tend_theta_euler_in": "tend_theta_euler"})
            if rk == 1 or (rk == 2 and stepper.order == 3):
                a = pop("vimp")
                gi = vimp_vjp(a, _route_out(acc, {PRE + c: c for c in COEFS}))
                _route_in(acc, gi, {"p": "exner", "t": "theta_m", "rt": "rtheta_p"})
        # the work fields start every RK stage from zero (small_step 1): nothing flows
        for k in WORK:
            acc.take(k)
    for save, src in SAVES:  # atm_rk_integration_setup
        acc.add(src, acc.take(save))
    pop("moist")
    assert not rec, [r[0] for r in rec]
    return {k: acc[k] for k in CARRIED if k in acc}


def prepare_vjp(stepper, st, dt, g):
    """Reverse mode of the cold-start preparation (Stepper.prepare): cotangents of the
    prepared fields (CARRIED names) -> cotangents of the loaded primitives u, w, theta,
    rho (dry)."""
    m, nc, ne, nl = stepper.m, stepper.nc, stepper.ne, stepper.nl
    prep, rec = _tape(stepper, stepper.prepare, st, dt)
    from .step import STAGE_NAMES
    names = {v: k for k, v in STAGE_NAMES.items()}
    rec = [(names[n], a) for n, a in rec]
    acc = _Acc()
    for k, v in g.items():
        acc.add("h_edge" if k == "rho_edge" else k, v)
    k_, a = rec.pop()
    assert k_ == "reconstruct"
    k_, a = rec.pop()
    assert k_ == "diag"
    gi = diag_vjp(a, _route_out(acc, {"h_edge": "h_edge", "v": "v", "divergence": "divergence",
                                      "vorticity": "vorticity", "ke": "ke", "pv_edge": "pv_edge"}))
    _route_in(acc, gi, {"u": "u", "h": "rho_zz"})
    zz = m["zz"][:nc]
    rb, tb = m["rho_base"][:nc], m["theta_base"][:nc]
    rho_zz = prep["rho_zz"][:nc]
    theta_m = prep["theta_m"][:nc]
    rho_p, rtp = prep["rho_p"][:nc], prep["rtheta_p"][:nc]
    ex = prep["exner"][:nc]
    rtb = prep["rtheta_base"][:nc]
    rcv = RGAS / (CP - RGAS)
    z = lambda k: (acc.take(k) if k in acc else np.zeros((nc + 1, nl)))[:nc]
    g_pp, g_ex, g_rtp, g_rho_p, g_th_m = z("pressure_p"), z("exner"), z("rtheta_p"), z("rho_p"), z("theta_m")
    g_rz = z("rho_zz").copy()
    g_ex = g_ex + g_pp * zz * RGAS * (rtp + rtb)
    g_rtp = g_rtp + g_pp * zz * RGAS * ex
    E = zz * (RGAS / P0) * (rtp + rtb)
    g_rtp = g_rtp + g_ex * rcv * ex / E * zz * (RGAS / P0)
    g_th_m = g_th_m + g_rtp * (rho_p + rb)
    g_rho_p = g_rho_p + g_rtp * theta_m
    g_rz += g_rho_p
    # rw (interior) = w rho_i zz_i + the slope terms (below)
    fzm, fzp = m["fzm"][:nl], m["fzp"][:nl]
    g_rw = z("rw")
    rho_i = fzp[None, 1:] * rho_zz[:, :nl - 1] + fzm[None, 1:] * rho_zz[:, 1:]
    zz_i = fzp[None, 1:] * zz[:, :nl - 1] + fzm[None, 1:] * zz[:, 1:]
    g_w = np.zeros((nc + 1, nl + 1))
    g_w[:nc] = z("w")
    g_w[:nc, 1:nl] += g_rw[:, 1:nl] * rho_i * zz_i
    g_rho_i = g_rw[:, 1:nl] * st["w"][:nc, 1:nl] * zz_i
    g_rz[:, 1:] += fzm[None, 1:] * g_rho_i
    g_rz[:, :nl - 1] += fzp[None, 1:] * g_rho_i
    # the slope terms of rw: - sum_j s_j (zb + sgn(flux_j) zb3) flux_j zz_i, flux_j = fzm
    # ru[k] + fzp ru[k-1] of the prepared ru (the selection held fixed)
    g_ru_slope = np.zeros((ne + 1, nl))
    eoc = S.idx0(m["edgesOnCell"][:nc], ne)
    n_eoc = np.asarray(m["nEdgesOnCell"][:nc]).astype(np.int64)
    sign = m["edgesOnCell_sign"][:nc]
    zb, zb3 = m["zb_cell"], m["zb3_cell"]
    ru_pad = np.concatenate([prep["ru"][:ne], np.zeros((1, nl))])
    for j in range(eoc.shape[1]):
        valid = (j < n_eoc) & (eoc[:, j] < ne)
        e = np.where(valid, eoc[:, j], ne)
        rs = ru_pad[e]
        flux = fzm[1:] * rs[:, 1:nl] + fzp[1:] * rs[:, :nl - 1]
        coef = zb[:nc, j, 1:nl] + _sgn(flux) * zb3[:nc, j, 1:nl]
        g_fl = np.where(valid[:, None], -g_rw[:, 1:nl] * sign[:, j, None] * coef * zz_i, 0.0)
        np.add.at(g_ru_slope, (e, slice(1, nl)), fzm[1:] * g_fl)
        np.add.at(g_ru_slope, (e, slice(0, nl - 1)), fzp[1:] * g_fl)
    # ru = 0.5 u (rho_1 + rho_2)
    coe = S.idx0(m["cellsOnEdge"][:ne], nc)
    u = st["u"]
    rz_pad = np.concatenate([rho_zz, np.zeros((1, nl))])
    g_ru = (acc.take("ru") if "ru" in acc else np.zeros((ne + 1, nl)))[:ne] + g_ru_slope[:ne]
    g_u = np.zeros((ne + 1, nl))
    g_u[:ne] = (acc.take("u") if "u" in acc else np.zeros((ne + 1, nl)))[:ne]
    g_u[:ne] += g_ru * 0.5 * (rz_pad[coe[:, 0]] + rz_pad[coe[:, 1]])
    gz = np.zeros((nc + 1, nl))
    np.add.at(gz, coe[:, 0], g_ru * 0.5 * u[:ne])
    np.add.at(gz, coe[:, 1], g_ru * 0.5 * u[:ne])
    g_rz += gz[:nc]
    qv = st["qv"][:nc] if "qv" in st else np.zeros((nc, nl))
    g_theta = np.zeros((nc + 1, nl))
    g_theta[:nc] = g_th_m * (1.0 + (461.6 / 287.0) * qv)
    g_rho = np.zeros((nc + 1, nl))
    g_rho[:nc] = g_rz / zz
    return {"u": g_u, "w": g_w, "theta": g_theta, "rho": g_rho}


def run_vjp(stepper, st0, dt, nsteps, g_final):
    """Cotangents of the loaded primitives (u, w, theta, rho) for cotangents of the state
    after ``nsteps`` large steps: preparation, then the steps, each checkpointed at its
    start and recomputed in the reverse sweep."""
    states = [stepper.prepare(st0, dt)]
    for _ in range(nsteps):
        states.append(stepper.srk3_step(states[-1], dt))
    g = dict(g_final)
    for n in range(nsteps - 1, -1, -1):
        g = step_vjp(stepper, states[n], dt, g)
    return prepare_vjp(stepper, st0, dt, g), states[-1]
