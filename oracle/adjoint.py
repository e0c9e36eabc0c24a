"""Oracle (test infrastructure): numpy restatement of the column tridiagonal operators
and their derivatives, as the reference states them in its serial form:
TridiagonalSolve (mpas_pytorch/autodiff/tridiagonal_solve.py:50-66 forward, :232-291
reverse, :294-352 forward mode) and TridiagonalFactorize (autodiff/tridiagonal_factor.py:17
forward, :183-231 reverse, :233-278 forward mode).  Pinned against vectors the reference
itself produced (tests/golden/make_golden_diag.py -> tridiag_ref.npz).

Also the derivatives of the hydrostatic surface-pressure diagnostic
(mpas_pytorch/diagnostics.py:77-86) with respect to rho_zz, qv, pressure_p and
pressure_base, and of the area-weighted squared-anomaly objective built on it, in the
order torch's reverse and forward modes evaluate the reference's expression; pinned
against vectors the reference produced (tests/golden/make_golden_sp_ad.py ->
sp_ad_g2.npz)."""

from __future__ import annotations

import numpy as np


def solve(a, al, g, rhs):
    L = a.shape[1]
    out = rhs.copy()
    for k in range(1, L):
        out[:, k] = (out[:, k] - a[:, k] * out[:, k - 1]) * al[:, k]
    for k in range(L - 1, -1, -1):
        out[:, k] = out[:, k] - g[:, k] * out[:, k + 1]
    return out


def solve_vjp(a, al, g, rhs, out, gout):
    L = a.shape[1]
    ga, gal, gg, gr = (np.zeros_like(a), np.zeros_like(al), np.zeros_like(g), np.zeros_like(rhs))
    adj_out = gout.copy()
    adj_u = np.zeros_like(rhs)
    for k in range(L):
        adj_u[:, k] += adj_out[:, k]
        gg[:, k] -= adj_out[:, k] * out[:, k + 1]
        adj_out[:, k + 1] -= g[:, k] * adj_out[:, k]
    adj_u[:, L] += adj_out[:, L]
    u = rhs.copy()
    for k in range(1, L):
        u[:, k] = (u[:, k] - a[:, k] * u[:, k - 1]) * al[:, k]
    for k in range(L - 1, 0, -1):
        t = rhs[:, k] - a[:, k] * u[:, k - 1]
        gal[:, k] += adj_u[:, k] * t
        adj_t = adj_u[:, k] * al[:, k]
        gr[:, k] += adj_t
        ga[:, k] -= adj_t * u[:, k - 1]
        adj_u[:, k - 1] -= adj_t * a[:, k]
    gr[:, 0] += adj_u[:, 0]
    gr[:, L] += adj_u[:, L]
    return ga, gal, gg, gr


def solve_jvp(a, al, g, rhs, out, da, dal, dg, dr):
    L = a.shape[1]
    u = rhs.copy()
    for k in range(1, L):
        u[:, k] = (u[:, k] - a[:, k] * u[:, k - 1]) * al[:, k]
    du = np.zeros_like(rhs)
    du[:, 0] = dr[:, 0]
    du[:, L] = dr[:, L]
    for k in range(1, L):
        t = rhs[:, k] - a[:, k] * u[:, k - 1]
        dt = dr[:, k] - da[:, k] * u[:, k - 1] - a[:, k] * du[:, k - 1]
        du[:, k] = dt * al[:, k] + t * dal[:, k]
    d = du.copy()
    for k in range(L - 1, -1, -1):
        d[:, k] = d[:, k] - dg[:, k] * out[:, k + 1] - g[:, k] * d[:, k + 1]
    return d


def factor(a, b, c):
    n, L = a.shape
    al, g = np.zeros((n, L)), np.zeros((n, L))
    for k in range(1, L):
        al[:, k] = 1.0 / (b[:, k] - a[:, k] * g[:, k - 1])
        g[:, k] = c[:, k] * al[:, k]
    return al, g


def factor_vjp(a, c, al, g, gal, gg):
    L = a.shape[1]
    ga, gb, gc = np.zeros_like(a), np.zeros_like(a), np.zeros_like(a)
    adj_g = gg.copy()
    for k in range(L - 1, 0, -1):
        gc[:, k] += adj_g[:, k] * al[:, k]
        tot = gal[:, k] + adj_g[:, k] * c[:, k]
        d_adj = -tot * (al[:, k] * al[:, k])
        gb[:, k] += d_adj
        ga[:, k] -= d_adj * g[:, k - 1]
        adj_g[:, k - 1] -= d_adj * a[:, k]
    return ga, gb, gc


def factor_jvp(a, c, al, g, da, db, dc):
    n, L = a.shape
    dal, dg = np.zeros((n, L)), np.zeros((n, L))
    for k in range(1, L):
        term = db[:, k] - da[:, k] * g[:, k - 1] - a[:, k] * dg[:, k - 1]
        dal[:, k] = -(al[:, k] * al[:, k]) * term
        dg[:, k] = dc[:, k] * al[:, k] + c[:, k] * dal[:, k]
    return dal, dg


GRAVITY = 9.80616


def _sp_geometry(nCells, zgrid, gravity):
    c = int(nCells)
    tem1 = zgrid[:c, 1] - zgrid[:c, 0]
    tem2 = zgrid[:c, 2] - zgrid[:c, 1]
    return c, tem1, tem1 + tem2, 0.5 * gravity * tem1


def surface_pressure_vjp(nCells, rho_zz, zz, qv, zgrid, g_sp, gravity=GRAVITY):
    """Cotangents of rho_zz, qv, pressure_p, pressure_base for the cotangent g_sp of the
    surface pressure (diagnostics.py:77-82 read backwards: hyd = A * B,
    B = rho1 - ((0.5 * (rho2 - rho1)) * tem1) / s); every level but 0 and 1 and the
    padding row get zero."""
    c, tem1, s, A = _sp_geometry(nCells, zgrid, gravity)
    out = {k: np.zeros_like(rho_zz) for k in ("rho_zz", "qv", "pressure_p", "pressure_base")}
    g = g_sp[:c]
    gB = g * A
    gD = 0.5 * ((-gB / s) * tem1)
    g_rho = (gB - gD, gD)
    for k in (0, 1):
        gr = g_rho[k]
        out["rho_zz"][:c, k] = (gr * (1.0 + qv[:c, k])) * zz[:c, k]
        out["qv"][:c, k] = gr * (rho_zz[:c, k] * zz[:c, k])
    out["pressure_p"][:c, 0] = g
    out["pressure_base"][:c, 0] = g
    return out


def surface_pressure_jvp(nCells, rho_zz, zz, qv, zgrid, t_rho_zz, t_qv, t_pressure_p, t_pressure_base,
                         gravity=GRAVITY):
    """Tangent of the surface pressure (padding row, when given, zero) for tangents of
    rho_zz, qv, pressure_p, pressure_base."""
    c, tem1, s, A = _sp_geometry(nCells, zgrid, gravity)
    d = [(t_rho_zz[:c, k] * zz[:c, k]) * (1.0 + qv[:c, k]) + (rho_zz[:c, k] * zz[:c, k]) * t_qv[:c, k]
         for k in (0, 1)]
    dC = ((0.5 * (d[1] - d[0])) * tem1) / s
    sp_t = A * (d[0] - dC) + t_pressure_p[:c, 0] + t_pressure_base[:c, 0]
    return np.concatenate([sp_t, np.zeros(rho_zz.shape[0] - c)])


def weighted_sq_sum_vjp(x, ref, weight, g_out=1.0):
    """Gradient of sum_i weight_i (x_i - ref_i)^2 with respect to x (ref's is its negative)."""
    d = x - (0.0 if ref is None else ref)
    return 2.0 * ((g_out * (1.0 if weight is None else weight)) * d)
