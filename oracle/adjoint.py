"""Oracle (test infrastructure): numpy restatement of the column tridiagonal operators
and their derivatives, as the reference states them in its serial form:
TridiagonalSolve (mpas_pytorch/autodiff/tridiagonal_solve.py:50-66 forward, :232-291
reverse, :294-352 forward mode) and TridiagonalFactorize (autodiff/tridiagonal_factor.py:17
forward, :183-231 reverse, :233-278 forward mode).  Pinned against vectors the reference
itself produced (tests/golden/make_golden_diag.py -> tridiag_ref.npz)."""

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
