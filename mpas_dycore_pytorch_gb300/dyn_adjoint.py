"""Reverse and forward mode of the dynamics through whole large steps (the reference's
``run_simulation.vjp`` / ``.jvp`` with respect to the dynamics state,
atmosphere_model.py:2101 / :2041).

``DynamicsAdjoint(model)`` holds, beside the model's own device state, a second device
state of the same layout for the cotangents, the transposed connectivity of the mesh, the
derivatives' work buffer and the per-step tape.  ``run_vjp`` runs the forward from the
loaded primitives with one checkpoint of the step boundary per large step in HBM (the
reference's per-step checkpoint, autodiff/checkpoint.py:106-254), then, from the last step
back, restores each step's checkpoint and runs ``mpasg_step_vjp`` (the step recomputed with
its tape, then its stages backwards: hand-written CUDA kernels, deterministic gathers), and
finally ``mpasg_prepare_vjp`` for the cold-start preparation.

``DynamicsTangent(model)`` holds the tangent state; ``run_jvp`` prepares the loaded
primitives with their tangents (``mpasg_prepare_jvp``) and advances values and tangents
together through every step (``mpasg_step_jvp``: each stage's forward and its hand-written
tangent kernels), with nothing stored.

Supported: float64 (and, in reverse mode, the mixed form), dry columns, flat or
terrain-following levels (the slope terms' upwind selections held fixed, as torch
differentiates sign), ``2d_smagorinsky`` or ``2d_fixed`` mixing with or without del4, vertical mixing of u, w and
theta (of the full state or of the perturbation from the initial profiles), CAM-style
top-level damping and Rayleigh damping of u, any RK order and substep counts; the objective
may read the step boundary's carried fields.  Everything else is
rejected before any device work with ``MpasUnsupportedCapabilityError``.
"""

from __future__ import annotations

import ctypes as C
from typing import Any, Callable, Mapping

import numpy as np
import torch

from . import _lib
from .errors import MpasConfigError, MpasNumericalError, MpasUnsupportedCapabilityError

# fields that carry derivatives from one large step to the next (a step's start state)
CARRIED = ("u", "v", "ru", "h_edge", "pv_edge", "w", "rw", "theta_m", "rho_zz", "rho_p", "rtheta_p", "exner",
           "pressure_p", "divergence", "ke", "vorticity")
# keys of run_simulation's output the objective may differentiate (rho_edge is h_edge)
DIFFERENTIABLE_OUT = CARRIED + ("rho_edge",)
# every field of the cotangent state the reverse-mode kernels read or write (the rest of the
# forward's fields are not allocated for it; a test checks this list against the sources)
COTANGENT_FIELDS = frozenset(CARRIED + (
    "ru_save", "rw_save", "rtheta_p_save", "rho_p_save", "theta_m_save", "rr_save", "theta_edge_save",
    "ru_p", "rw_p", "rho_pp", "rtheta_pp", "rtheta_pp_old", "ac_x",
    "tend_u", "tend_u_euler", "tend_w", "tend_w_euler", "tend_rw", "tend_theta", "tend_theta_euler", "tend_rho",
    "kdiff", "cofwz", "cofwt", "coftz", "a_tri", "alpha_tri", "gamma_tri"))
TRACKABLE = ("u", "w", "theta", "rho")


def _stream() -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t: torch.Tensor) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


def check_request(cfg: Mapping[str, Any], merged: Mapping[str, Any], num_scalars: int,
                  allow_mixed: bool = False) -> None:
    """The dynamics derivative's scope, checked on the host from the configuration and the
    mesh before any device work (the same limits as ``check_supported``).  The reverse mode
    also takes the mixed form (its trajectory, linearised in float64); the forward mode is
    float64 only."""
    from .device import _int, _np
    why = []
    prec = str(cfg.get("config_precision", "float64"))
    if prec != "float64" and not (allow_mixed and prec == "mixed"):
        why.append("float64 or mixed arithmetic (config_precision)" if allow_mixed
                   else "float64 arithmetic only (config_precision)")
    ms, me = _int(merged.get("moist_start", 1)), _int(merged.get("moist_end", num_scalars))
    if not me < ms:
        why.append("dry columns only (moist_end < moist_start)")
    if why:
        raise MpasUnsupportedCapabilityError("dynamics derivatives on the GB300 path: " + "; ".join(why))


def check_supported(model, allow_mixed: bool = False) -> None:
    """The dynamics derivative's scope (mpasg.h): raise before any derivative work."""
    cfg, cs, dm = model.cfg, model.cstruct, model.dmesh
    why = []
    if cs.precision != _lib.PRECISIONS["float64"] and not (allow_mixed and cs.precision == _lib.PRECISIONS["mixed"]):
        why.append("float64 arithmetic only (config_precision)")
    if not (cs.moist_end < cs.moist_start):
        why.append("dry columns only (moist_end < moist_start)")
    if model._perm is not None:
        why.append("native mesh order only")
    if why:
        raise MpasUnsupportedCapabilityError("dynamics derivatives on the GB300 path: " + "; ".join(why))
    del cfg


def transpose_tables(dmesh, mesh_ref: Mapping[str, Any]) -> dict[str, np.ndarray]:
    """The transposed connectivity the reverse-mode gathers read (mpasg_transpose)."""
    nc, ne, nv = dmesh.nCells, dmesh.nEdges, dmesh.nVertices
    me2, vd = dmesh.maxEdges2, dmesh.vertexDegree
    I = {k: np.asarray(v, dtype=np.int64) for k, v in dmesh.ints.items()}
    eoc, neoc, coe = I["edgesOnCell"], I["nEdgesOnCell"], I["cellsOnEdge"]
    eov, voe = I["edgesOnVertex"], I["verticesOnEdge"]
    eoe, neoe = I["edgesOnEdge"], I["nEdgesOnEdge"]
    voc, kite = I["verticesOnCell"], I["kiteForCell"]
    me = eoc.shape[1]
    edge_cell = np.full((ne, 2), -1, dtype=np.int64)
    cells = np.arange(nc)
    for j in range(me):
        ok = (j < neoc) & (eoc[:, j] < ne)
        e = eoc[ok, j]
        c = cells[ok]
        side = np.where(coe[e, 0] == c, 0, np.where(coe[e, 1] == c, 1, -1))
        good = side >= 0
        edge_cell[e[good], side[good]] = j
    edge_vert = np.full((ne, 2), -1, dtype=np.int64)
    verts = np.arange(nv)
    for j in range(vd):
        ok = eov[:, j] < ne
        e = eov[ok, j]
        v = verts[ok]
        side = np.where(voe[e, 0] == v, 0, np.where(voe[e, 1] == v, 1, -1))
        good = side >= 0
        edge_vert[e[good], side[good]] = j
    eoe_t = np.full((ne, me2), -1, dtype=np.int64)
    edges = np.arange(ne)
    for j in range(me2):
        ok = (j < neoe) & (eoe[:, j] < ne)
        e, eo = edges[ok], eoe[ok, j]
        for jt in range(me2):
            hit = (jt < neoe[eo]) & (eoe[eo, jt] == e) & (eoe_t[e, j] < 0)
            eoe_t[e[hit], j] = jt
    if "cellsOnVertex" in mesh_ref:
        cov_raw = np.asarray(mesh_ref["cellsOnVertex"].detach().cpu() if isinstance(mesh_ref["cellsOnVertex"], torch.Tensor)
                             else mesh_ref["cellsOnVertex"], dtype=np.int64)[:nv, :vd]
        cov = np.where((cov_raw >= 1) & (cov_raw <= nc), cov_raw - 1, nc)
    else:  # from verticesOnCell
        cov = np.full((nv, vd), nc, dtype=np.int64)
        fill = np.zeros(nv, dtype=np.int64)
        for c in range(nc):
            for j in range(int(neoc[c])):
                v = voc[c, j]
                if v < nv and fill[v] < vd:
                    cov[v, fill[v]] = c
                    fill[v] += 1
    vkite = np.full((nv, vd), -1, dtype=np.int64)
    for s in range(vd):
        c = cov[:, s]
        okc = c < nc
        cc = np.where(okc, c, 0)
        for j in range(me):
            hit = okc & (j < neoc[cc]) & (voc[cc, j] == verts) & (vkite[:, s] < 0)
            vkite[hit, s] = kite[cc[hit], j]
    from .tracer_adjoint import transport_adjacency
    adj = transport_adjacency(dmesh)
    return {"edgeCellSlot": edge_cell.astype(np.int32), "edgeVertexSlot": edge_vert.astype(np.int32),
            "eoeTransSlot": eoe_t.astype(np.int32), "cellsOnVertex": cov.astype(np.int32),
            "vertexKite": vkite.astype(np.int32),
            "advPtr": adj["adj_ptr"].cpu().numpy(), "advIdx": adj["adj_es"].cpu().numpy()}


class DynamicsAdjoint:
    """Cotangent state, transposed connectivity, work buffer and tape of one Model."""

    def __init__(self, model):
        from .device import DeviceState
        check_supported(model, allow_mixed=True)
        self.model = model
        self.lib = model.lib
        dm = model.dmesh
        dev = dm.device
        tabs = transpose_tables(dm, model.mesh_ref)
        self._tabs = {k: torch.as_tensor(np.ascontiguousarray(v), device=dev) for k, v in tabs.items()}
        t = _lib.TransposeStruct()
        for k in _lib.TRANSPOSE_PTRS:
            setattr(t, k, self._tabs[k].data_ptr())
        self.t = t
        self.g = DeviceState(dm, model.state.num_scalars, only=COTANGENT_FIELDS)
        self.g.f["rho_zz"].zero_()  # a cotangent: the padding sentinel does not apply
        self.window_tape: torch.Tensor | None = None
        n = int(self.lib.mpasg_dyn_vjp_work_doubles(C.byref(dm.struct)))
        self.work = torch.zeros(n, dtype=torch.float64, device=dev)
        self.tape: torch.Tensor | None = None
        self._graph = None
        self._warm = False

    # -- checkpoints of the step boundary -------------------------------------------
    def checkpoint(self) -> dict[str, torch.Tensor]:
        return {k: self.model.state.f[k].clone() for k in CARRIED}

    def restore(self, ck: Mapping[str, torch.Tensor]) -> None:
        for k in CARRIED:
            self.model.state.f[k].copy_(ck[k])

    def zero_cotangents(self) -> None:
        self.g.arena.zero_()

    def _tape(self) -> torch.Tensor:
        if self.tape is None:
            n = int(self.lib.mpasg_step_vjp_tape_doubles(C.byref(self.model.dmesh.struct),
                                                         C.byref(self.model.cstruct)))
            if n <= 0:
                raise MpasConfigError("mpasg_step_vjp_tape_doubles: invalid configuration")
            self.tape = torch.empty(n, dtype=torch.float64, device=self.model.dmesh.device)
        return self.tape

    # -- one step / preparation -----------------------------------------------------
    def _call_step_vjp(self, stream: C.c_void_p) -> int:
        m = self.model
        mp, cp, fp, gp = C.byref(m.dmesh.struct), C.byref(m.cstruct), C.byref(m.state.struct), C.byref(self.g.struct)
        tape = _p(self._tape())
        rc = self.lib.mpasg_step_tape(mp, cp, fp, tape, stream)
        if rc != 0:
            return rc
        return self.lib.mpasg_step_vjp_taped(mp, cp, fp, gp, C.byref(self.t), tape, _p(self.work), stream)

    def step_vjp(self) -> None:
        """Cotangents in g of the state after one step (from the state in the model) ->
        cotangents of the step's start state; the model's state ends one step later.  The
        first call runs eagerly (it also makes the kernels' one-time per-device settings);
        the second captures the step's tape and reverse pass as one CUDA graph, replayed by
        every later call (same buffers, so the graph stays valid)."""
        if self._graph is not None:
            self._graph.replay()
            return
        if not self._warm:
            _lib.check(self._call_step_vjp(_stream()), "mpasg_step_vjp")
            self._warm = True
            return
        torch.cuda.synchronize()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                rc = self._call_step_vjp(C.c_void_p(s.cuda_stream))
        _lib.check(rc, "mpasg_step_vjp (capture)")
        torch.cuda.current_stream().wait_stream(s)
        self._graph = g
        g.replay()

    def step_tape(self, tape: torch.Tensor) -> None:
        """One step of the model with its tape written to ``tape`` (no transport)."""
        m = self.model
        rc = self.lib.mpasg_step_tape(C.byref(m.dmesh.struct), C.byref(m.cstruct), C.byref(m.state.struct),
                                      _p(tape), _stream())
        _lib.check(rc, "mpasg_step_tape")

    def step_vjp_taped(self, tape: torch.Tensor) -> None:
        """The reverse pass of one step from its tape."""
        m = self.model
        rc = self.lib.mpasg_step_vjp_taped(C.byref(m.dmesh.struct), C.byref(m.cstruct), C.byref(m.state.struct),
                                           C.byref(self.g.struct), C.byref(self.t), _p(tape), _p(self.work),
                                           _stream())
        _lib.check(rc, "mpasg_step_vjp_taped")

    def step_vjp_window(self, sub: int) -> None:
        """The reverse pass of dynamics substep ``sub`` (1-based) of the step that starts at the
        model's state, with only that substep taped (mpasg_step_vjp_window); g holds the
        cotangents of the state after the substep on entry, before it on return."""
        m = self.model
        if self.window_tape is None:
            n = int(self.lib.mpasg_step_vjp_window_tape_doubles(C.byref(m.dmesh.struct), C.byref(m.cstruct), 1))
            if n <= 0:
                raise MpasConfigError("mpasg_step_vjp_window_tape_doubles: invalid configuration")
            self.window_tape = torch.empty(n, dtype=torch.float64, device=m.dmesh.device)
        rc = self.lib.mpasg_step_vjp_window(C.byref(m.dmesh.struct), C.byref(m.cstruct), C.byref(m.state.struct),
                                            C.byref(self.g.struct), C.byref(self.t), _p(self.window_tape),
                                            _p(self.work), int(sub), int(sub), _stream())
        _lib.check(rc, "mpasg_step_vjp_window")

    def tape_doubles(self) -> int:
        return int(self.lib.mpasg_step_vjp_tape_doubles(C.byref(self.model.dmesh.struct),
                                                        C.byref(self.model.cstruct)))

    def prepare_vjp(self, w_in: torch.Tensor) -> dict[str, torch.Tensor]:
        """Cotangents in g of the prepared state (the model holds it) -> cotangents of the
        loaded u, w, theta, rho."""
        m = self.model
        f = m.state.f
        out = {k: torch.empty_like(f[n]) for k, n in (("u", "u"), ("w", "w"), ("theta", "theta_m"),
                                                       ("rho", "rho_zz"))}
        rc = self.lib.mpasg_prepare_vjp(C.byref(m.dmesh.struct), C.byref(m.cstruct), C.byref(m.state.struct),
                                        C.byref(self.g.struct), C.byref(self.t), _p(w_in), _p(out["u"]),
                                        _p(out["w"]), _p(out["theta"]), _p(out["rho"]), _p(self.work), _stream())
        _lib.check(rc, "mpasg_prepare_vjp")
        return out


class VjpRun:
    """The two phases of a reverse-mode run, so that they can happen at different times
    (``run_vjp``; ``run_simulation(differentiable=True)`` runs the forward phase in its
    forward and the reverse phase when autograd asks for the inputs' gradients).

    ``forward()`` prepares the loaded primitives and runs ``nsteps`` large steps, keeping
    what the reverse phase needs under the checkpoint mode; it returns the final state.
    ``reverse(g)`` takes cotangents of the final state's carried fields (and ``rho_edge``)
    and returns those of the loaded u, w, theta, rho; it can run once.

    ``checkpoint="step"`` (the reference's default, checkpoint_timesteps on): one checkpoint
    of the step boundary per step in HBM; the reverse pass of each step first recomputes it
    with its tape.  ``checkpoint="none"`` (checkpoint_timesteps=False): every step's tape is
    kept from the forward pass (about ``tape_doubles() * 8 * nsteps`` bytes), nothing is
    recomputed; the forward then advances the dynamics only, so the final state's scalars
    and reconstructed winds are not part of it.  ``checkpoint="sqrt"`` (for meshes whose
    per-step checkpoints and whole-step tape do not fit): checkpoints every S = ceil(sqrt(
    nsteps)) steps; each segment is recomputed from its checkpoint with a checkpoint per step,
    and each step runs backwards one dynamics substep at a time, every substep recomputed
    from the step's checkpoint with only its own tape (mpasg_step_vjp_window).  Checkpoints
    held: at most ceil(nsteps / S) + S - 1; the same gradient bit for bit."""

    def __init__(self, model, loaded: Mapping[str, Any], nsteps: int, adj: DynamicsAdjoint | None = None,
                 checkpoint: str = "step"):
        if checkpoint not in ("step", "none", "sqrt"):
            raise MpasConfigError(f"checkpoint must be 'step', 'none' or 'sqrt', got {checkpoint!r}")
        self.model, self.loaded, self.nsteps, self.mode = model, loaded, int(nsteps), checkpoint
        self.adj = adj or DynamicsAdjoint(model)
        self.done = False

    def forward(self) -> dict:
        model, adj, nsteps, checkpoint = self.model, self.adj, self.nsteps, self.mode
        model.prepare(self.loaded)
        self.w_in = model.state.f["w"].clone()
        self.ck0 = adj.checkpoint()
        self.tapes: list[torch.Tensor | None] = []
        self.ckpts = [self.ck0]
        self.seg = max(1, int(np.ceil(np.sqrt(nsteps)))) if checkpoint == "sqrt" else 1
        self.outer = {0: self.ck0}

        def forward_step(n):
            model.step()
            if n == 0 and nsteps > 1 and model._graph is None:
                model.capture_graph()  # later steps replay the step graph (bitwise the eager step)

        if checkpoint == "step":
            for n in range(nsteps):
                forward_step(n)
                if n + 1 < nsteps:
                    self.ckpts.append(adj.checkpoint())
        elif checkpoint == "sqrt":
            for n in range(nsteps):
                forward_step(n)
                if n + 1 < nsteps and (n + 1) % self.seg == 0:
                    self.outer[n + 1] = adj.checkpoint()
        else:
            nd = adj.tape_doubles()
            free, _ = torch.cuda.mem_get_info(model.dmesh.device)
            if nd * 8 * nsteps > 0.9 * free:
                raise MpasConfigError(f"checkpoint='none' needs {nd * 8 * nsteps / 1e9:.1f} GB of tapes; "
                                      f"{free / 1e9:.1f} GB are free (use checkpoint='step')")
            for n in range(nsteps):
                self.tapes.append(torch.empty(nd, dtype=torch.float64, device=model.dmesh.device))
                adj.step_tape(self.tapes[-1])
        bad = model.check_finite()
        if bad:
            raise MpasNumericalError(f"forecast result contains {bad} nonfinite values")
        final = model.export()
        if checkpoint == "none":
            for k in ("scalars", "uReconstructX", "uReconstructY", "uReconstructZ", "uReconstructZonal",
                      "uReconstructMeridional", "ur_cell", "vr_cell"):
                final.pop(k, None)
        return final

    def reverse(self, g: Mapping[str, torch.Tensor]) -> dict:
        if self.done:
            raise MpasUnsupportedCapabilityError("the reverse pass of a derivative run can run once")
        self.done = True
        model, adj, nsteps, checkpoint = self.model, self.adj, self.nsteps, self.mode
        adj.zero_cotangents()
        dev = model.dmesh.device
        for k, v in g.items():
            name = "h_edge" if k == "rho_edge" else k
            if name not in CARRIED:
                raise MpasUnsupportedCapabilityError(f"no derivative through output {k!r}")
            dst = adj.g.f[name]
            dst[: v.shape[0]].add_(v.to(device=dev, dtype=torch.float64))
        if checkpoint == "sqrt":
            split = int(model.cstruct.dynamics_split_steps)
            seg, outer = self.seg, self.outer
            for start in sorted(outer, reverse=True):
                end = min(start + seg, nsteps)
                adj.restore(outer[start])
                inner = [outer[start]]
                for n in range(start, end - 1):
                    model.step()
                    inner.append(adj.checkpoint())
                for n in range(end - 1, start - 1, -1):
                    for sub in range(split, 0, -1):
                        adj.restore(inner[n - start])
                        adj.step_vjp_window(sub)
                if start > 0:
                    del outer[start]
                del inner
        else:
            for n in range(nsteps - 1, -1, -1):
                if checkpoint == "step":
                    adj.restore(self.ckpts[n])
                    adj.step_vjp()
                else:
                    adj.step_vjp_taped(self.tapes[n])
                    self.tapes[n] = None  # free as the sweep goes
        self.ckpts = []
        adj.restore(self.ck0)
        return adj.prepare_vjp(self.w_in)


def run_vjp(model, loaded: Mapping[str, Any], nsteps: int,
            cotangents: Callable[[dict], Mapping[str, torch.Tensor]],
            adj: DynamicsAdjoint | None = None, checkpoint: str = "step") -> tuple[dict, dict]:
    """Forward from the loaded primitives through ``nsteps`` large steps, then the reverse
    sweep (``VjpRun``, which describes the checkpoint modes).  ``cotangents(out)`` receives
    the final state (the model's export) and returns cotangents of some of its carried
    fields.  Returns the cotangents of the loaded u, w, theta, rho and the final state."""
    run = VjpRun(model, loaded, nsteps, adj, checkpoint)
    final = run.forward()
    return run.reverse(cotangents(final)), final


class DynamicsTangent:
    """Tangent state and work buffer of one Model (forward mode)."""

    def __init__(self, model):
        from .device import DeviceState
        check_supported(model)
        self.model = model
        self.lib = model.lib
        dm = model.dmesh
        self.d = DeviceState(dm, model.state.num_scalars)
        self.d.arena.zero_()
        self.work = torch.zeros((dm.nCells + 1) * (dm.nVertLevels + 1), dtype=torch.float64, device=dm.device)

    def _args(self):
        m = self.model
        return C.byref(m.dmesh.struct), C.byref(m.cstruct), C.byref(m.state.struct), C.byref(self.d.struct)

    def prepare_jvp(self, dtheta: torch.Tensor | None, drho: torch.Tensor | None) -> None:
        """Tangents of the prepared state (the model holds it) from the tangents of the loaded
        u and w (already in the tangent state) and of theta and rho."""
        rc = self.lib.mpasg_prepare_jvp(*self._args(), _p(dtheta) if dtheta is not None else C.c_void_p(0),
                                        _p(drho) if drho is not None else C.c_void_p(0), _stream())
        _lib.check(rc, "mpasg_prepare_jvp")

    def step_jvp(self) -> None:
        """One step of the model's dynamics with the tangents alongside."""
        _lib.check(self.lib.mpasg_step_jvp(*self._args(), _p(self.work), _stream()), "mpasg_step_jvp")


def run_jvp(model, loaded: Mapping[str, Any], nsteps: int, perturbation: Mapping[str, torch.Tensor],
            tan: DynamicsTangent | None = None) -> dict[str, torch.Tensor]:
    """Tangents of the final carried fields (and ``rho_edge``) along ``perturbation`` of the
    loaded u, w, theta, rho (rows as loaded; padding rows are not perturbed), through the
    preparation and ``nsteps`` large steps.  The model's state ends with the dynamics of the
    final step (its scalars are not advanced)."""
    tan = tan or DynamicsTangent(model)
    dev = model.dmesh.device
    model.prepare(loaded)
    d = tan.d.f
    tan.d.arena.zero_()

    def device_copy(key, shape):
        v = perturbation.get(key)
        if v is None:
            return None
        out = torch.zeros(shape, dtype=torch.float64, device=dev)
        rows = min(int(v.shape[0]), shape[0] - 1)  # the padding row stays unperturbed
        out[:rows] = v[:rows].to(device=dev, dtype=torch.float64)
        return out

    for key in ("u", "w"):
        t = device_copy(key, tuple(d[key].shape))
        if t is not None:
            d[key].copy_(t)
    dth = device_copy("theta", tuple(d["theta_m"].shape))
    drho = device_copy("rho", tuple(d["rho_zz"].shape))
    tan.prepare_jvp(dth, drho)
    for _ in range(int(nsteps)):
        tan.step_jvp()
    bad = model.check_finite()
    if bad:
        raise MpasNumericalError(f"forecast result contains {bad} nonfinite values")
    out = {k: d["h_edge" if k == "rho_edge" else k].clone() for k in DIFFERENTIABLE_OUT}
    for k, v in out.items():
        if not bool(torch.isfinite(v).all()):
            raise MpasNumericalError(f"tangent of {k!r} contains nonfinite values")
    return out
