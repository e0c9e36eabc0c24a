"""Diagnostics derived from the dynamics state, on the GPU.

``physics_interface_surface_pressure`` mirrors the reference's function of the same name
(mpas_pytorch/diagnostics.py:10): same keyword arguments, shape checks and error
messages; the arithmetic runs in ``mpasg_surface_pressure`` (bit-exact float64).
``surface_pressure_functional`` is the area-weighted squared surface-pressure anomaly
used as the scalar objective of the differentiation checks (``mpasg_weighted_sq_sum``,
fixed summation order).

Both are differentiable like the reference's, whose autograd differentiates the torch
expression: with ``rho_zz``, ``qv``, ``pressure_p`` or ``pressure_base`` requiring grad
(or carrying forward-mode tangents) the surface pressure runs through a
``torch.autograd.Function`` whose backward is ``mpasg_surface_pressure_vjp`` and whose
forward-mode rule is ``mpasg_surface_pressure_jvp``, both bit-identical to torch's
derivatives of the reference's expression; the objective's backward is
``mpasg_weighted_sq_sum_vjp`` (with respect to ``sp`` and ``sp_ref``).  Derivatives with
respect to the mesh inputs (``zz``, ``zgrid``) and the weights (``area``) are not built and
are rejected before any device work.
"""

from __future__ import annotations

import ctypes as C

import torch
import torch.autograd.forward_ad as fwAD

from . import _lib
from .errors import MpasUnsupportedCapabilityError

GRAVITY = 9.80616


def _dev(t: torch.Tensor, name: str) -> torch.Tensor:
    if not isinstance(t, torch.Tensor) or t.device.type != "cuda":
        raise ValueError(f"{name} must be a CUDA tensor")
    return t.to(torch.float64).contiguous()


def physics_interface_surface_pressure(*, nCells: int, rho_zz: torch.Tensor, zz: torch.Tensor, qv: torch.Tensor,
                                       pressure_p: torch.Tensor, pressure_base: torch.Tensor, zgrid: torch.Tensor,
                                       gravity: float = GRAVITY) -> torch.Tensor:
    """Hydrostatic surface pressure (Pa), one value per input cell row (padding row 0)."""
    fields = {"rho_zz": rho_zz, "zz": zz, "qv": qv, "pressure_p": pressure_p,
              "pressure_base": pressure_base, "zgrid": zgrid}
    for name, value in fields.items():
        if value.ndim != 2:
            raise ValueError(f"{name} must be rank-2, got shape {tuple(value.shape)}")
    if rho_zz.shape[0] not in (nCells, nCells + 1):
        raise ValueError(f"rho_zz first dimension must be nCells ({nCells}) or nCells+1 "
                         f"({nCells + 1}), got {rho_zz.shape[0]}")
    state_shape = tuple(rho_zz.shape)
    for name in ("zz", "qv", "pressure_p", "pressure_base"):
        if tuple(fields[name].shape) != state_shape:
            raise ValueError(f"{name} shape {tuple(fields[name].shape)} does not match rho_zz {state_shape}")
    if zgrid.shape[0] != rho_zz.shape[0]:
        raise ValueError(f"zgrid cell extent must match rho_zz: {zgrid.shape[0]} != {rho_zz.shape[0]}")
    if rho_zz.shape[1] < 2 or zgrid.shape[1] < 3:
        raise ValueError("surface pressure requires two mass levels and three W levels")
    if zgrid.shape[1] != rho_zz.shape[1] + 1:
        raise ValueError("zgrid must have one more level than rho_zz")
    for name in ("zz", "zgrid"):
        if fields[name].requires_grad or _has_tangent(fields[name]):
            raise MpasUnsupportedCapabilityError(
                f"surface-pressure derivatives with respect to the mesh input {name} are not built")
    return _SurfacePressure.apply(int(nCells), float(gravity), rho_zz, zz, qv, pressure_p, pressure_base, zgrid)


def _has_tangent(x: torch.Tensor) -> bool:
    """True when x carries a forward-mode tangent at the current dual level."""
    return fwAD.unpack_dual(x).tangent is not None


def _ptr(x: torch.Tensor | None) -> C.c_void_p:
    return C.c_void_p(x.data_ptr()) if x is not None else C.c_void_p(0)


def _stream(x: torch.Tensor) -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream(x.device).cuda_stream)


class _SurfacePressure(torch.autograd.Function):
    """Surface pressure with hand-written reverse and forward derivatives."""

    @staticmethod
    def forward(ctx, nCells, gravity, rho_zz, zz, qv, pressure_p, pressure_base, zgrid):
        lib = _lib.load()
        t = [_dev(v, k) for k, v in (("rho_zz", rho_zz), ("zz", zz), ("qv", qv), ("pressure_p", pressure_p),
                                       ("pressure_base", pressure_base), ("zgrid", zgrid))]
        rows, nlev = int(rho_zz.shape[0]), int(rho_zz.shape[1])
        out = torch.empty(rows, dtype=torch.float64, device=t[0].device)
        rc = lib.mpasg_surface_pressure(nCells, rows, nlev, *[_ptr(x) for x in t], gravity, _ptr(out), _stream(out))
        _lib.check(rc, "mpasg_surface_pressure")
        ctx.nCells, ctx.gravity = nCells, gravity
        base = (t[0], t[1], t[2], t[5])  # rho_zz, zz, qv, zgrid as float64 contiguous
        ctx.save_for_backward(*base)
        ctx.save_for_forward(*base)
        return out

    @staticmethod
    def backward(ctx, g_sp):
        rho_zz, zz, qv, zgrid = ctx.saved_tensors
        need = ctx.needs_input_grad
        rows, nlev = int(rho_zz.shape[0]), int(rho_zz.shape[1])
        g_sp = g_sp.to(torch.float64).contiguous()
        outs = [torch.empty(rows, nlev, dtype=torch.float64, device=rho_zz.device) if need[i] else None
                for i in (2, 4, 5, 6)]
        rc = _lib.load().mpasg_surface_pressure_vjp(ctx.nCells, rows, nlev, _ptr(rho_zz), _ptr(zz), _ptr(qv),
                                                    _ptr(zgrid), ctx.gravity, _ptr(g_sp), *[_ptr(o) for o in outs],
                                                    _stream(rho_zz))
        _lib.check(rc, "mpasg_surface_pressure_vjp")
        return None, None, outs[0], None, outs[1], outs[2], outs[3], None

    @staticmethod
    def jvp(ctx, _n, _g, t_rho_zz, _t_zz, t_qv, t_pressure_p, t_pressure_base, _t_zgrid):
        # zz / zgrid tangents are zeros torch materialises (dual mesh inputs are rejected
        # before apply)
        rho_zz, zz, qv, zgrid = ctx.saved_tensors
        rows, nlev = int(rho_zz.shape[0]), int(rho_zz.shape[1])
        tan = [None if x is None else _dev(x, "tangent") for x in (t_rho_zz, t_qv, t_pressure_p, t_pressure_base)]
        out = torch.empty(rows, dtype=torch.float64, device=rho_zz.device)
        rc = _lib.load().mpasg_surface_pressure_jvp(ctx.nCells, rows, nlev, _ptr(rho_zz), _ptr(zz), _ptr(qv),
                                                    _ptr(zgrid), ctx.gravity, *[_ptr(x) for x in tan], _ptr(out),
                                                    _stream(out))
        _lib.check(rc, "mpasg_surface_pressure_jvp")
        return out


class _WeightedSqSum(torch.autograd.Function):
    """sum_i w_i (x_i - r_i)^2 with a hand-written backward for x and r."""

    @staticmethod
    def forward(ctx, x, r, w):
        out = torch.empty((), dtype=torch.float64, device=x.device)
        rc = _lib.load().mpasg_weighted_sq_sum(int(x.numel()), _ptr(x), _ptr(r), _ptr(w), _ptr(out), _stream(x))
        _lib.check(rc, "mpasg_weighted_sq_sum")
        ctx.save_for_backward(x, r, w)
        return out

    @staticmethod
    def backward(ctx, g_out):
        x, r, w = ctx.saved_tensors
        need = ctx.needs_input_grad
        g_x = torch.empty_like(x) if need[0] else None
        g_r = torch.empty_like(x) if need[1] else None
        g_out = g_out.to(torch.float64).contiguous()
        rc = _lib.load().mpasg_weighted_sq_sum_vjp(int(x.numel()), _ptr(x), _ptr(r), _ptr(w), _ptr(g_out),
                                                   _ptr(g_x), _ptr(g_r), _stream(x))
        _lib.check(rc, "mpasg_weighted_sq_sum_vjp")
        return g_x, g_r, None


def surface_pressure_functional(sp: torch.Tensor, sp_ref: torch.Tensor | None, area: torch.Tensor | None,
                                nCells: int) -> torch.Tensor:
    """sum_c area_c (sp_c - sp_ref_c)^2 over the active cells (0-d float64 CUDA tensor)."""
    if area is not None and area.requires_grad:
        raise MpasUnsupportedCapabilityError("objective derivatives with respect to area are not built")
    x = _dev(sp, "sp")[:nCells].contiguous()
    r = _dev(sp_ref, "sp_ref")[:nCells].contiguous() if sp_ref is not None else None
    w = _dev(area, "area")[:nCells].contiguous() if area is not None else None
    return _WeightedSqSum.apply(x, r, w)
