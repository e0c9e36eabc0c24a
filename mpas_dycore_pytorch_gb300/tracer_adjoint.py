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
the ``scalars`` key in that case.  In the coupled transport mode (one dynamics substep:
the scalars advance inside every RK stage with that stage's fluxes and density) the
step runs through ``mpasg_step_taped``, which records each stage's transport inputs, and
the adjoint runs stage by stage (``mpasg_transport_vjp_stage``).  The monotone limiter
and moist scalars (whose derivatives run through the dynamics) are rejected.
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
    if not _flag(cfg, "config_scalar_advection"):
        bad.append("config_scalar_advection = false")
    if moist_end >= moist_start:
        bad.append("moist scalars (their derivatives run through the dynamics)")
    if bad:
        raise MpasUnsupportedCapabilityError(
            "scalar derivatives on the GB300 path cover the explicit transport of passive scalars; "
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


def is_coupled(model) -> bool:
    """One dynamics substep: the scalars advance inside every RK stage."""
    return int(model.cstruct.dynamics_split_steps) == 1


def _dts(model) -> tuple[float, float, float]:
    """The transport stage timesteps (time_integration.py:3366-3370; the coupled mode's
    rk_timestep with one dynamics substep is the same)."""
    dt = float(model.cstruct.dt)
    return (dt / 2.0 if int(model.cstruct.time_integration_order) == 2 else dt / 3.0, dt / 2.0, dt)


class ScalarTape:
    """Each step's transport inputs: in the split mode the step's averaged mass fluxes
    and its start and end densities, recorded after the step from the model's fields; in
    the coupled mode every RK stage's fluxes and density (``mpasg_step_taped``) and the
    step's start density."""

    def __init__(self, model=None):
        self.steps: list[dict] = []
        self.coupled = model is not None and is_coupled(model)
        self._buf = None
        if self.coupled:
            dm = model.dmesh
            C, E, L = dm.nCells, dm.nEdges, dm.nVertLevels
            self._sizes = ((E + 1) * L, (C + 1) * (L + 1), (C + 1) * L)
            self._shapes = ((E + 1, L), (C + 1, L + 1), (C + 1, L))
            self._buf = torch.empty(3 * sum(self._sizes), dtype=torch.float64, device=dm.device)

    def step(self, model) -> None:
        """Run one large step of ``model`` and record its transport inputs."""
        if self.coupled:
            model.call("mpasg_step_taped", C.c_void_p(self._buf.data_ptr()))
            buf = self._buf.clone()
            stages, off = [], 0
            for _ in range(3):
                parts = []
                for n, shp in zip(self._sizes, self._shapes):
                    parts.append(buf[off:off + n].view(shp))
                    off += n
                stages.append(tuple(parts))
            self.steps.append({"stages": stages, "rho_zz_old_split": model.state.f["rho_zz_old_split"].clone()})
        else:
            model.step()
            self.record(model)

    def record(self, model) -> None:
        self.steps.append({k: model.state.f[k].clone() for k in TAPE_KEYS})


def scalars_vjp(model, tape: ScalarTape, g_end: torch.Tensor) -> torch.Tensor:
    """Cotangent of the start scalars of the taped steps (device order, (C+1, L, S))."""
    lib = _lib.load()
    dm = model.dmesh
    adj = transport_adjacency(dm)
    L, S = dm.nVertLevels, int(model.cstruct.num_scalars)
    ncs, nes = (dm.nCells + 1) * L * S, (dm.nEdges + 1) * L * S
    g = g_end.to(torch.float64).contiguous().clone()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if tape.coupled:
        return _coupled_vjp(lib, model, tape, adj, g, stream)
    work = torch.empty(3 * ncs + nes, dtype=torch.float64, device=g_end.device)
    out = torch.empty_like(g)
    for rec in reversed(tape.steps):
        rc = lib.mpasg_transport_vjp(C.byref(dm.struct), C.byref(model.cstruct), _p(rec["ruAvg"]), _p(rec["wwAvg"]),
                                     _p(rec["rho_zz_old_split"]), _p(rec["rho_zz"]), _p(adj["adj_ptr"]),
                                     _p(adj["adj_es"]), _p(adj["edge_cell_w"]), _p(g), _p(out), _p(work), stream)
        _lib.check(rc, "mpasg_transport_vjp")
        g, out = out, g
    return g


def _coupled_vjp(lib, model, tape: ScalarTape, adj, g: torch.Tensor, stream) -> torch.Tensor:
    """The coupled mode's adjoint: per step in reverse, the three stages in reverse, each
    with its own fluxes and density (weights w_old = 0, w_new = 1); the cotangent of the
    step's start is the stage-1 input cotangent plus the accumulated s_old cotangents."""
    dm = model.dmesh
    nc = dm.nCells
    L, S = dm.nVertLevels, int(model.cstruct.num_scalars)
    work_e = torch.empty((dm.nEdges + 1) * L * S, dtype=torch.float64, device=g.device)
    dts = _dts(model)
    for rec in reversed(tape.steps):
        gold = torch.zeros_like(g)
        cur = g
        for rk in (3, 2, 1):
            ru, ww, rho = rec["stages"][rk - 1]
            sbar = torch.zeros_like(g)
            rc = lib.mpasg_transport_vjp_stage(C.byref(dm.struct), C.byref(model.cstruct), C.c_double(dts[rk - 1]),
                                               C.c_double(0.0), C.c_double(1.0), _p(ru), _p(ww),
                                               _p(rec["rho_zz_old_split"]), _p(rho), _p(adj["adj_ptr"]),
                                               _p(adj["adj_es"]), _p(adj["edge_cell_w"]), _p(cur), _p(sbar),
                                               _p(gold), _p(work_e), stream)
            _lib.check(rc, "mpasg_transport_vjp_stage")
            cur = sbar
        start = gold + cur
        start[nc:] = g[nc:]  # the padding row passes through the step unchanged
        g = start
    return g


def scalars_jvp(model, tape: ScalarTape, v_start: torch.Tensor) -> torch.Tensor:
    """Tangent of the end scalars of the taped steps along v_start (device order): the
    library's explicit transport stages replayed on the tangent with each step's fluxes."""
    lib = _lib.load()
    dm = model.dmesh
    c = model.cstruct
    dts = _dts(model)
    v0 = v_start.to(torch.float64).contiguous().clone()
    a, b = torch.zeros_like(v0), torch.zeros_like(v0)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for rec in tape.steps:
        f = _lib.FieldsStruct.from_buffer_copy(model.state.struct)
        if not tape.coupled:
            f.ruAvg, f.wwAvg = rec["ruAvg"].data_ptr(), rec["wwAvg"].data_ptr()
            f.rho_zz = rec["rho_zz"].data_ptr()
        f.rho_zz_old_split = rec["rho_zz_old_split"].data_ptr()
        a.copy_(v0)
        f.scalars_init = v0.data_ptr()
        for rk in (1, 2, 3):
            if tape.coupled:  # this stage's fluxes and density
                ru, ww, rho = rec["stages"][rk - 1]
                f.ruAvg, f.wwAvg, f.rho_zz = ru.data_ptr(), ww.data_ptr(), rho.data_ptr()
            f.scalars_a, f.scalars_b = a.data_ptr(), b.data_ptr()
            rc = lib.mpasg_advance_scalars(C.byref(dm.struct), C.byref(c), C.byref(f), rk, C.c_double(dts[rk - 1]),
                                           stream)
            _lib.check(rc, "mpasg_advance_scalars (tangent)")
            a, b = b, a
        pad = v0[dm.nCells:].clone()  # the padding row passes through the step unchanged
        v0 = a.clone()
        v0[dm.nCells:] = pad
    return v0
