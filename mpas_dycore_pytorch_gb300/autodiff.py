"""Hand-written derivatives on the GPU: ``TridiagonalSolve`` and ``TridiagonalFactorize``.

``torch.autograd.Function`` classes with the reference's names and contracts
(mpas_pytorch/autodiff/tridiagonal_solve.py:177, autodiff/tridiagonal_factor.py:145):
forward, ``backward`` (VJP) and ``jvp`` are CUDA kernels (``mpasg_tridiag_*``, one thread
per column, float64).  Inputs must be CUDA tensors.
"""

from __future__ import annotations

import ctypes as C
from typing import Any

import torch

from . import _lib


def _p(t: torch.Tensor | None) -> C.c_void_p:
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


def _stream(t: torch.Tensor) -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


def _prep(*ts: torch.Tensor | None) -> list[torch.Tensor | None]:
    out = []
    for t in ts:
        if t is None:
            out.append(None)
            continue
        if t.device.type != "cuda":
            raise ValueError("the GB300 tridiagonal operators take CUDA tensors")
        out.append(t.detach().to(torch.float64).contiguous())
    return out


def _check_solve_shapes(a, alpha, gamma, rhs) -> None:
    if a.shape != alpha.shape or a.shape != gamma.shape:
        raise ValueError("a_tri, alpha_tri, gamma_tri must have identical shapes")
    if a.ndim != 2:
        raise ValueError("expected tridiagonal tensors with shape (nCells, nVertLevels)")
    if rhs.ndim != 2 or rhs.shape[0] != a.shape[0] or rhs.shape[1] != a.shape[1] + 1:
        raise ValueError("rhs must have shape (nCells, nVertLevels + 1)")


class TridiagonalSolve(torch.autograd.Function):
    """out = solve(a_tri, alpha_tri, gamma_tri, rhs); rhs (and out) have one more level
    than the factors (the boundary value used by the back substitution)."""

    @staticmethod
    def forward(ctx: Any, a_tri, alpha_tri, gamma_tri, rhs):
        _check_solve_shapes(a_tri, alpha_tri, gamma_tri, rhs)
        a, al, g, r = _prep(a_tri, alpha_tri, gamma_tri, rhs)
        n, L = a.shape
        out = torch.empty_like(r)
        rc = _lib.load().mpasg_tridiag_solve(n, L, _p(a), _p(al), _p(g), _p(r), _p(out), _stream(out))
        _lib.check(rc, "mpasg_tridiag_solve")
        ctx.save_for_backward(a, al, g, r, out)
        ctx.save_for_forward(a, al, g, r, out)
        return out

    @staticmethod
    def backward(ctx: Any, grad_out):
        a, al, g, r, out = ctx.saved_tensors
        (go,) = _prep(grad_out)
        n, L = a.shape
        ga, gal, gg, gr = torch.empty_like(a), torch.empty_like(al), torch.empty_like(g), torch.empty_like(r)
        rc = _lib.load().mpasg_tridiag_solve_vjp(n, L, _p(a), _p(al), _p(g), _p(r), _p(out), _p(go), _p(ga),
                                                 _p(gal), _p(gg), _p(gr), _stream(out))
        _lib.check(rc, "mpasg_tridiag_solve_vjp")
        return ga, gal, gg, gr

    @staticmethod
    def jvp(ctx: Any, da, dal, dg, dr):
        a, al, g, r, out = ctx.saved_tensors
        da, dal, dg, dr = _prep(da, dal, dg, dr)
        n, L = a.shape
        dout = torch.empty_like(out)
        rc = _lib.load().mpasg_tridiag_solve_jvp(n, L, _p(a), _p(al), _p(g), _p(r), _p(out), _p(da), _p(dal),
                                                 _p(dg), _p(dr), _p(dout), _stream(out))
        _lib.check(rc, "mpasg_tridiag_solve_jvp")
        return dout


class TridiagonalFactorize(torch.autograd.Function):
    """(alpha_tri, gamma_tri) = factorize(a_tri, b_tri, c_tri), the Thomas factors."""

    @staticmethod
    def forward(ctx: Any, a_tri, b_tri, c_tri):
        if a_tri.shape != b_tri.shape or a_tri.shape != c_tri.shape or a_tri.ndim != 2:
            raise ValueError("a_tri, b_tri, c_tri must be (nCells, nVertLevels) tensors of one shape")
        a, b, c = _prep(a_tri, b_tri, c_tri)
        n, L = a.shape
        al, g = torch.empty_like(a), torch.empty_like(a)
        rc = _lib.load().mpasg_tridiag_factor(n, L, _p(a), _p(b), _p(c), _p(al), _p(g), _stream(a))
        _lib.check(rc, "mpasg_tridiag_factor")
        ctx.save_for_backward(a, c, al, g)
        ctx.save_for_forward(a, c, al, g)
        return al, g

    @staticmethod
    def backward(ctx: Any, grad_alpha, grad_gamma):
        a, c, al, g = ctx.saved_tensors
        gal = torch.zeros_like(al) if grad_alpha is None else _prep(grad_alpha)[0]
        gg = torch.zeros_like(g) if grad_gamma is None else _prep(grad_gamma)[0]
        n, L = a.shape
        ga, gb, gc = torch.empty_like(a), torch.empty_like(a), torch.empty_like(a)
        rc = _lib.load().mpasg_tridiag_factor_vjp(n, L, _p(a), _p(c), _p(al), _p(g), _p(gal), _p(gg), _p(ga),
                                                  _p(gb), _p(gc), _stream(a))
        _lib.check(rc, "mpasg_tridiag_factor_vjp")
        return ga, gb, gc

    @staticmethod
    def jvp(ctx: Any, da, db, dc):
        a, c, al, g = ctx.saved_tensors
        da, db, dc = _prep(da, db, dc)
        n, L = a.shape
        dal, dg = torch.empty_like(al), torch.empty_like(g)
        rc = _lib.load().mpasg_tridiag_factor_jvp(n, L, _p(a), _p(c), _p(al), _p(g), _p(da), _p(db), _p(dc),
                                                  _p(dal), _p(dg), _stream(a))
        _lib.check(rc, "mpasg_tridiag_factor_jvp")
        return dal, dg


def tridiagonal_solve(a_tri, alpha_tri, gamma_tri, rhs):
    return TridiagonalSolve.apply(a_tri, alpha_tri, gamma_tri, rhs)


def tridiagonal_factorize(a_tri, b_tri, c_tri):
    return TridiagonalFactorize.apply(a_tri, b_tri, c_tri)
