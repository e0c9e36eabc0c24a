"""Hand-written derivatives of large steps with respect to the transported scalars.

With no moist species among the scalars (moist_end < moist_start) the dynamics never
read the scalars, and the split transport maps a step's start scalars linearly to its end
scalars given the step's averaged mass fluxes and densities.  So through any number of
steps:

* the JVP (tangent of the end scalars along a perturbation of the start scalars) is the
  same transport applied to the perturbation, replayed by the library's own transport
  kernels with each step's recorded fluxes;
* the VJP (cotangent of the start scalars) runs the transposed transport of every step
  in reverse (``mpasg_transport_vjp``: edge and cell gathers, no atomics).

Both are exact for the explicit (non-monotone) transport stages, which is what the
reference's ``run_simulation.jvp`` / ``.vjp`` (atmosphere_model.py:2041, :2101) return for
the ``scalars`` key in that case.  The monotone limiter, coupled transport and moist
scalars (whose derivatives run through the dynamics) are rejected.
"""

from __future__ import annotations

import ctypes as C
from typing import Any, Mapping

import numpy as np
import torch

from . import _lib
from .errors import MpasUnsupportedCapabilityError

TAPE_KEYS = ("ruAvg", "wwAvg", "rho_zz_old_split", "rho_zz")


def _p(t: torch.Tensor) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


def check_supported(cfg: Mapping[str, Any], moist_start: int, moist_end: int) -> None:
    from .api import _flag
    bad = []
    if _flag(cfg, "config_monotonic") or _flag(cfg, "config_positive_definite"):
        bad.append("the monotone limiter (config_monotonic / config_positive_definite)")
    if not _flag(cfg, "config_split_dynamics_transport") or int(cfg["config_dynamics_split_steps"]) < 2:
        bad.append("coupled transport")
    if not _flag(cfg, "config_scalar_advection"):
        bad.append("config_scalar_advection = false")
    if moist_end >= moist_start:
        bad.append("moist scalars (their derivatives run through the dynamics)")
    if bad:
        raise MpasUnsupportedCapabilityError(
            "scalar derivatives on the GB300 path cover the explicit split transport of passive scalars; "
            f"unsupported here: {bad}")


def transport_adjacency(dmesh) -> dict[str, torch.Tensor]:
    """The advection stencils transposed (cell -> its (edge, slot) readers, CSR in edge
    order) and each edge's two cell weights -sign * invAreaCell, on the device."""
    cached = getattr(dmesh, "_transport_adjacency", None)
    if cached is not None:
        return cached
    nc, ne = dmesh.nCells, dmesh.nEdges
    na = dmesh.nAdvMax
    adv = np.asarray(dmesh.ints["advCellsForEdge"], dtype=np.int64)[:ne, :na]
    nadv = np.asarray(dmesh.ints["nAdvCellsForEdge"], dtype=np.int64)[:ne]
    slot = np.arange(na)[None, :]
    valid = (slot < nadv[:, None]) & (adv >= 0) & (adv < nc)
    cells = adv[valid]
    es = (np.arange(ne)[:, None] * na + slot)[valid]
    order = np.lexsort((es, cells))  # by cell, then edge * nAdvMax + slot
    cells, es = cells[order], es[order]
    ptr = np.zeros(nc + 1, dtype=np.int64)
    np.add.at(ptr, cells + 1, 1)
    ptr = np.cumsum(ptr)
    coe = np.asarray(dmesh.ints["cellsOnEdge"], dtype=np.int64)[:ne]
    eoc = np.asarray(dmesh.ints["edgesOnCell"], dtype=np.int64)[:nc]
    neoc = np.asarray(dmesh.ints["nEdgesOnCell"], dtype=np.int64)[:nc]
    sign = dmesh._keep["edgesOnCell_sign"].cpu().numpy()[:nc]
    inv_area = dmesh._keep["invAreaCell"].cpu().numpy()
    w = np.zeros((ne, 2))
    for j in range(eoc.shape[1]):
        ok = j < neoc
        for side in (0, 1):
            c = coe[:, side]
            act = c < nc
            cc = np.where(act, c, 0)
            hit = act & ok[cc] & (eoc[cc, j] == np.arange(ne))
            w[hit, side] = -sign[cc[hit], j] * inv_area[cc[hit]]
    dev = dmesh.device
    out = {"adj_ptr": torch.as_tensor(ptr.astype(np.int32), device=dev),
           "adj_es": torch.as_tensor(es.astype(np.int32), device=dev),
           "edge_cell_w": torch.as_tensor(np.ascontiguousarray(w), device=dev)}
    dmesh._transport_adjacency = out
    return out


class ScalarTape:
    """Each step's transport inputs (averaged mass fluxes, start and end densities),
    recorded after the step from the model's fields."""

    def __init__(self):
        self.steps: list[dict[str, torch.Tensor]] = []

    def record(self, model) -> None:
        self.steps.append({k: model.state.f[k].clone() for k in TAPE_KEYS})


def scalars_vjp(model, tape: ScalarTape, g_end: torch.Tensor) -> torch.Tensor:
    """Cotangent of the start scalars of the taped steps (device order, (C+1, L, S))."""
    lib = _lib.load()
    dm = model.dmesh
    adj = transport_adjacency(dm)
    L, S = dm.nVertLevels, int(model.cstruct.num_scalars)
    ncs, nes = (dm.nCells + 1) * L * S, (dm.nEdges + 1) * L * S
    work = torch.empty(3 * ncs + nes, dtype=torch.float64, device=g_end.device)
    g = g_end.to(torch.float64).contiguous().clone()
    out = torch.empty_like(g)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for rec in reversed(tape.steps):
        rc = lib.mpasg_transport_vjp(C.byref(dm.struct), C.byref(model.cstruct), _p(rec["ruAvg"]), _p(rec["wwAvg"]),
                                     _p(rec["rho_zz_old_split"]), _p(rec["rho_zz"]), _p(adj["adj_ptr"]),
                                     _p(adj["adj_es"]), _p(adj["edge_cell_w"]), _p(g), _p(out), _p(work), stream)
        _lib.check(rc, "mpasg_transport_vjp")
        g, out = out, g
    return g


def scalars_jvp(model, tape: ScalarTape, v_start: torch.Tensor) -> torch.Tensor:
    """Tangent of the end scalars of the taped steps along v_start (device order): the
    library's explicit transport stages replayed on the tangent with each step's fluxes."""
    lib = _lib.load()
    dm = model.dmesh
    c = model.cstruct
    dt = float(c.dt)
    order = int(c.time_integration_order)
    dts = (dt / 2.0 if order == 2 else dt / 3.0, dt / 2.0, dt)
    v0 = v_start.to(torch.float64).contiguous().clone()
    a, b = torch.zeros_like(v0), torch.zeros_like(v0)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for rec in tape.steps:
        f = _lib.FieldsStruct.from_buffer_copy(model.state.struct)
        f.ruAvg, f.wwAvg = rec["ruAvg"].data_ptr(), rec["wwAvg"].data_ptr()
        f.rho_zz_old_split, f.rho_zz = rec["rho_zz_old_split"].data_ptr(), rec["rho_zz"].data_ptr()
        a.copy_(v0)
        f.scalars_init = v0.data_ptr()
        for rk in (1, 2, 3):
            f.scalars_a, f.scalars_b = a.data_ptr(), b.data_ptr()
            rc = lib.mpasg_advance_scalars(C.byref(dm.struct), C.byref(c), C.byref(f), rk, C.c_double(dts[rk - 1]),
                                           stream)
            _lib.check(rc, "mpasg_advance_scalars (tangent)")
            a, b = b, a
        pad = v0[dm.nCells:].clone()  # the padding row passes through the step unchanged
        v0 = a.clone()
        v0[dm.nCells:] = pad
    return v0
