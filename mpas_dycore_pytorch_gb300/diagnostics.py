"""Diagnostics derived from the dynamics state, on the GPU.

``physics_interface_surface_pressure`` mirrors the reference's function of the same name
(mpas_pytorch/diagnostics.py:10): same keyword arguments, shape checks and error
messages; the arithmetic runs in ``mpasg_surface_pressure`` (bit-exact float64).
``surface_pressure_functional`` is the area-weighted squared surface-pressure anomaly
used as the scalar objective of the differentiation checks (``mpasg_weighted_sq_sum``,
fixed summation order).
"""

from __future__ import annotations

import ctypes as C

import torch

from . import _lib

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
    lib = _lib.load()
    t = {k: _dev(v, k) for k, v in fields.items()}
    rows = int(rho_zz.shape[0])
    out = torch.empty(rows, dtype=torch.float64, device=t["rho_zz"].device)
    p = lambda x: C.c_void_p(x.data_ptr())
    rc = lib.mpasg_surface_pressure(int(nCells), rows, int(rho_zz.shape[1]), p(t["rho_zz"]), p(t["zz"]), p(t["qv"]),
                                    p(t["pressure_p"]), p(t["pressure_base"]), p(t["zgrid"]), float(gravity), p(out),
                                    C.c_void_p(torch.cuda.current_stream(out.device).cuda_stream))
    _lib.check(rc, "mpasg_surface_pressure")
    return out


def surface_pressure_functional(sp: torch.Tensor, sp_ref: torch.Tensor | None, area: torch.Tensor | None,
                                nCells: int) -> torch.Tensor:
    """sum_c area_c (sp_c - sp_ref_c)^2 over the active cells (0-d float64 CUDA tensor)."""
    lib = _lib.load()
    x = _dev(sp, "sp")[:nCells].contiguous()
    r = _dev(sp_ref, "sp_ref")[:nCells].contiguous() if sp_ref is not None else None
    w = _dev(area, "area")[:nCells].contiguous() if area is not None else None
    out = torch.empty((), dtype=torch.float64, device=x.device)
    ptr = lambda v: C.c_void_p(v.data_ptr()) if v is not None else C.c_void_p(0)
    rc = lib.mpasg_weighted_sq_sum(int(nCells), ptr(x), ptr(r), ptr(w), ptr(out),
                                   C.c_void_p(torch.cuda.current_stream(x.device).cuda_stream))
    _lib.check(rc, "mpasg_weighted_sq_sum")
    return out
