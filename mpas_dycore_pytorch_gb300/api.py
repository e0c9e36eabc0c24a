"""Reference-facing API of the GB300 step: ``run_simulation``, ``run_timestep``, ``atm_srk3``
and the per-stage ``atm_*_work`` operators.

Names, argument meaning and error types follow the reference
(mpas_pytorch/atmosphere_model.py:900 ``run_timestep``, :1474 ``run_simulation``;
dynamics/time_integration.py:4897 ``atm_srk3``; stage functions as listed in
``STAGES``).  State and mesh dictionaries use the reference's padded layout and key
names; returned tensors live on the CUDA device.  There is no CPU path: the reference
itself is the CPU implementation.
"""

from __future__ import annotations

import ctypes as C
import math
from typing import Any, Callable, Mapping

import numpy as np
import torch

from . import _lib
from .device import DeviceMesh, DeviceState, STATE_KEYS, _int, _np
from .boundary import (MARKER, has_complete_step_boundary, mark_complete_step_boundary,
                       require_boundary_continuation_identity, require_unedited_boundary_support)
from .errors import MpasConfigError, MpasDeviceError, MpasNumericalError, MpasUnsupportedCapabilityError

DEFAULTS = {
    "config_time_integration_order": 2, "config_number_of_sub_steps": 2,
    "config_dynamics_split_steps": 3, "config_split_dynamics_transport": True,
    "config_epssm": 0.1, "config_smdiv": 0.1, "config_len_disp": 0.0,
    "config_visc4_2dsmag": 0.05, "config_del4u_div_factor": 10.0,
    "config_apvm_upwinding": 0.5, "config_horiz_mixing": "2d_smagorinsky",
    "config_monotonic": True, "config_positive_definite": False, "config_scalar_advection": True,
    "config_h_mom_eddy_visc2": 0.0, "config_h_mom_eddy_visc4": 0.0,
    "config_v_mom_eddy_visc2": 0.0, "config_h_theta_eddy_visc2": 0.0,
    "config_h_theta_eddy_visc4": 0.0, "config_v_theta_eddy_visc2": 0.0,
    "config_rayleigh_damp_u": False, "config_rayleigh_damp_u_timescale_days": 5.0,
    "config_number_rayleigh_damp_u_levels": 6,
    "config_mpas_cam_coef": 0.0, "config_number_cam_damping_levels": 4,
    "config_curvature_u": False, "config_mix_full": True, "config_IAU_option": "off",
    "config_apply_lbcs": False, "config_dt": 720.0,
    # GB300 extension (no reference counterpart): "float64" (the reference's arithmetic)
    # or "mixed" (float32 horizontal stencils over float64 state, see include/mpasg.h)
    "config_precision": "float64",
    # the reference's RCM option (atmosphere_model.py:810-827): results in the RCM order
    "config_mesh_reordering_rcm": False,
}


def resolved_config(config: Mapping[str, Any] | None) -> dict:
    cfg = dict(DEFAULTS)
    cfg.update(config or {})
    return cfg


_TRUE = {"1", "true", "t", "yes", "y", "on", ".true.", ".t."}
_FALSE = {"0", "false", "f", "no", "n", "off", "", ".false.", ".f."}
# logical namelist switches whose true value asks for a mode outside the dycore
# (restart, data assimilation, surface updates, decomposition, regional boundaries)
_UNSUPPORTED_SWITCHES = ("config_do_restart", "config_do_DAcycling", "config_jedi_da", "config_sst_update",
                         "config_sstdiurn_update", "config_deepsoiltemp_update", "config_explicit_proc_decomp",
                         "config_apply_lbcs", "config_enable_sharding")


def _logical(value: Any, key: str) -> bool:
    """A namelist logical: Python / numpy / torch booleans and numbers, or Fortran-style
    strings ("true", ".true.", "t", "off", ...); anything else is a configuration error."""
    if hasattr(value, "item") and callable(value.item):
        value = value.item()
    if isinstance(value, str):
        v = value.strip().lower()
        if v in _TRUE:
            return True
        if v in _FALSE:
            return False
        raise MpasConfigError(f"{key}: expected a logical value, got {value!r}")
    return bool(value)


def _flag(cfg: Mapping[str, Any], key: str) -> bool:
    return _logical(cfg[key], key)


def active_unsupported_settings(cfg: Mapping[str, Any]) -> list[str]:
    """Keys of ``cfg`` that request a mode this path does not run (a physics suite, a
    physics scheme, IAU, restart / assimilation / surface-update switches, sharding,
    regional boundaries), with the reference's reading of their values
    (namelist_metadata.py:76-106)."""
    bad = []
    norm = lambda v: str(v).strip().lower()
    if norm(cfg.get("config_physics_suite", "none")) not in ("", "none", "off"):
        bad.append("config_physics_suite")
    if norm(cfg.get("config_IAU_option", "off")) not in ("", "off", "none"):
        bad.append("config_IAU_option")
    for key in _UNSUPPORTED_SWITCHES:
        short = key[len("config_"):]
        if key in cfg or short in cfg:
            if _logical(cfg[key] if key in cfg else cfg[short], key):
                bad.append(key)
    for key in sorted(cfg):
        if isinstance(key, str) and key.startswith("config_") and key.endswith("_scheme") and \
                norm(cfg[key]) not in ("", "none", "off"):
            bad.append(key)
    return bad


def reject_unsupported_request(state: Mapping[str, Any] | None, mesh: Mapping[str, Any] | None,
                               config: Mapping[str, Any] | None) -> None:
    """The public routes' first check, before any preparation or device work: unsupported
    modes and reduced-precision float storage (the reference's
    tests/test_configuration_contracts.py:48-80 contract)."""
    bad = active_unsupported_settings(config or {})
    if bad:
        raise MpasUnsupportedCapabilityError(f"unsupported active MPAS settings on the GB300 path: {bad}")
    for where, d in (("state", state), ("mesh", mesh)):
        for key, v in (d or {}).items():
            dt = getattr(v, "dtype", None)
            if dt is None:
                continue
            if dt in (torch.float32, torch.float16, torch.bfloat16) or \
                    (isinstance(dt, np.dtype) and dt.kind == "f" and dt.itemsize < 8):
                raise MpasUnsupportedCapabilityError(
                    f"{where}[{key!r}] has dtype {dt}; the GB300 path takes float64 storage "
                    "(config_precision selects the arithmetic)")


FINITE_CHECK_KEYS = ("u", "w", "theta", "rho", "theta_m", "rho_zz", "scalars", "qv", "rho_base", "theta_base",
                     "zz", "pressure_p", "pressure_base")


def require_finite_inputs(state: Mapping[str, Any], context: str = "initial state") -> None:
    """Reject non-finite model fields before any work (the reference's check,
    atmosphere_model.py:77-94), as MpasNumericalError (an MpasConfigError)."""
    for name in FINITE_CHECK_KEYS:
        v = state.get(name)
        if isinstance(v, torch.Tensor):
            if v.is_floating_point() and not bool(torch.isfinite(v).all()):
                raise MpasNumericalError(f"{context}: {name} contains nonfinite values")
        elif isinstance(v, np.ndarray) and v.dtype.kind == "f" and not np.all(np.isfinite(v)):
            raise MpasNumericalError(f"{context}: {name} contains nonfinite values")


def validate_supported(cfg: Mapping[str, Any]) -> None:
    """Reject options outside the implemented path before any device work (mirrors the
    reference's capability rejection, tests/test_configuration_contracts.py:48-79)."""
    bad = active_unsupported_settings(cfg)
    if int(cfg["config_dynamics_split_steps"]) < 1:
        bad.append("config_dynamics_split_steps < 1")
    if int(cfg["config_time_integration_order"]) not in (2, 3):
        bad.append("config_time_integration_order")
    if _flag(cfg, "config_curvature_u"):
        bad.append("config_curvature_u")
    if str(cfg["config_horiz_mixing"]) not in ("2d_smagorinsky", "2d_fixed"):
        bad.append("config_horiz_mixing")
    if str(cfg["config_precision"]) not in _lib.PRECISIONS:
        bad.append("config_precision")
    if bad:
        raise MpasUnsupportedCapabilityError(f"unsupported on the GB300 path: {bad}")


def resolve_len_disp(cfg: Mapping[str, Any], mesh: Mapping[str, Any]) -> float:
    """config_len_disp, else nominalMinDc, else the minimum dcEdge (time_integration.py:1882)."""
    ld = float(cfg.get("config_len_disp", 0.0))
    if ld > 0.0:
        return ld
    if "nominalMinDc" in mesh and float(_np(mesh["nominalMinDc"]).reshape(-1)[0]) > 0.0:
        return float(_np(mesh["nominalMinDc"]).reshape(-1)[0])
    ne = _int(mesh["nEdges"])
    return float(np.min(_np(mesh["dcEdge"])[:ne]))


def make_config(cfg: Mapping[str, Any], mesh: Mapping[str, Any], dt: float, num_scalars: int,
                moist_start: int, moist_end: int) -> _lib.ConfigStruct:
    c = _lib.ConfigStruct()
    c.dt = float(dt)
    c.epssm = float(cfg["config_epssm"])
    c.smdiv = float(cfg["config_smdiv"])
    c.len_disp = resolve_len_disp(cfg, mesh)
    c.coef_3rd_order = float(_np(mesh.get("coef_3rd_order", cfg.get("config_coef_3rd_order", 0.25))).reshape(-1)[0])
    c.c_s = float(_np(mesh.get("c_s", cfg.get("config_smagorinsky_coef", 0.125))).reshape(-1)[0])
    c.visc4_2dsmag = float(cfg["config_visc4_2dsmag"])
    c.del4u_div_factor = float(cfg["config_del4u_div_factor"])
    c.apvm_upwinding = float(cfg["config_apvm_upwinding"])
    c.h_mom_eddy_visc4 = float(cfg["config_h_mom_eddy_visc4"])
    c.h_theta_eddy_visc4 = float(cfg["config_h_theta_eddy_visc4"])
    c.time_integration_order = int(cfg["config_time_integration_order"])
    c.number_of_sub_steps = int(cfg["config_number_of_sub_steps"])
    # split transport off is one dynamics substep with the scalars inside the RK stages
    # (the reference's _resolve_dynamics_split, time_integration.py:1809-1878)
    c.dynamics_split_steps = int(cfg["config_dynamics_split_steps"]) if _flag(cfg, "config_split_dynamics_transport") else 1
    # the positive-definite option selects the same limited final transport stage
    # (time_integration.py:3979-3987)
    c.monotonic = 1 if (_flag(cfg, "config_monotonic") or _flag(cfg, "config_positive_definite")) else 0
    c.horiz_mixing_smagorinsky = 1 if str(cfg["config_horiz_mixing"]) == "2d_smagorinsky" else 0
    c.num_scalars = int(num_scalars)
    c.moist_start = int(moist_start)
    c.moist_end = int(moist_end)
    c.precision = _lib.PRECISIONS[str(cfg["config_precision"])]
    c.h_theta_eddy_visc2 = float(cfg["config_h_theta_eddy_visc2"])
    c.v_mom_eddy_visc2 = float(cfg["config_v_mom_eddy_visc2"])
    c.v_theta_eddy_visc2 = float(cfg["config_v_theta_eddy_visc2"])
    c.mpas_cam_coef = float(cfg["config_mpas_cam_coef"])
    c.number_cam_damping_levels = int(cfg["config_number_cam_damping_levels"])
    c.scalar_advection_off = 0 if _flag(cfg, "config_scalar_advection") else 1
    c.rayleigh_damp_u_timescale_days = float(cfg["config_rayleigh_damp_u_timescale_days"])
    c.rayleigh_damp_u_levels = int(cfg["config_number_rayleigh_damp_u_levels"]) if _flag(cfg, "config_rayleigh_damp_u") else 0
    c.mix_perturbation = 0 if _flag(cfg, "config_mix_full") else 1
    return c


# boundary fields written by the second part of a step (mpasg_step_part 1), and those a
# step never writes (base state and diabatic forcing, set by the preparation)
LATE_KEYS = ("scalars",)
STATIC_KEYS = ("rtheta_base", "exner_base", "pressure_base", "rt_diabatic_tend")


def _copy_stream(device) -> torch.cuda.Stream:
    """A stream for the host copies of a step boundary, at the highest priority: with a
    reordered mesh every field copied out or in passes through a row gather (a kernel),
    and at the default priority those gathers queue behind the blocks of the step's own
    kernels, so the copies of a step's result stall while the next kernels run (measured:
    1.6 ms more per level-6 step through ``run_host``)."""
    return torch.cuda.Stream(device=device, priority=-1)


def _stream_ptr(stream: torch.cuda.Stream | None = None) -> C.c_void_p:
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


class Model:
    """One mesh + configuration + timestep resident on a GPU: the native step and its state."""

    def __init__(self, mesh: Mapping[str, Any], config: Mapping[str, Any] | None, dt: float,
                 num_scalars: int | None = None, device: str | torch.device = "cuda",
                 precision: str | None = None, order: str = "native"):
        """``order="sfc"`` keeps the mesh and state on the device in Hilbert-curve order
        (``reorder.py``); inputs and ``export()`` stay in the caller's order."""
        self.lib = _lib.load()
        if order not in ("native", "sfc"):
            raise MpasConfigError(f"order must be 'native' or 'sfc', got {order!r}")
        self._perm = None
        if order == "sfc":
            from .reorder import apply_permutation, compute_sfc_permutation
            self._dims = tuple(_int(mesh[k]) for k in ("nCells", "nEdges", "nVertices"))
            self._perm = compute_sfc_permutation(mesh)
            mesh = apply_permutation(mesh, self._perm, self._dims)
        self.cfg = resolved_config(config)
        if precision is not None:
            self.cfg["config_precision"] = precision
        validate_supported(self.cfg)
        if not (math.isfinite(float(dt)) and float(dt) > 0.0):
            raise MpasConfigError("dt must be positive and finite")
        self.dt = float(dt)
        device = torch.device(device)
        if device.type != "cuda":
            raise MpasUnsupportedCapabilityError("the GB300 path runs on CUDA devices only")
        if not torch.cuda.is_available():
            raise MpasDeviceError("no CUDA device is available")
        self.mesh_ref = mesh
        self.dmesh = DeviceMesh(mesh, device)
        if self.dmesh.nVertLevels < 4:
            raise MpasConfigError("at least 4 vertical levels are required")
        ns = int(num_scalars if num_scalars is not None else _int(mesh.get("num_scalars", 1)))
        self.state = DeviceState(self.dmesh, ns)
        self.moist_start = _int(mesh.get("moist_start", 1))
        self.moist_end = _int(mesh.get("moist_end", ns))
        self.cstruct = make_config(self.cfg, mesh, self.dt, ns, self.moist_start, self.moist_end)
        # static fields the step reads from the state side
        self.state.load(mesh, keys=("rt_diabatic_tend",))
        self._graph = None
        self._graph_parts = None
        self._d2h_stream = self._h2d_stream = None
        self._pending_d2h: dict[int, torch.cuda.Event] = {}
        self._rows_in = self._rows_out = None
        if self._perm is not None:  # device row maps, padding row last
            dev = self.dmesh.device
            idx = lambda a, n: torch.as_tensor(np.concatenate([a, [n]]).astype(np.int64), device=dev)
            nc, ne, nv = self._dims
            self._rows_in = {"cell": idx(self._perm.cell_new_to_old, nc), "edge": idx(self._perm.edge_new_to_old, ne),
                             "vertex": idx(self._perm.vertex_new_to_old, nv)}
            self._rows_out = {"cell": idx(self._perm.cell_old_to_new, nc), "edge": idx(self._perm.edge_old_to_new, ne),
                              "vertex": idx(self._perm.vertex_old_to_new, nv)}

    # -- C ABI plumbing ---------------------------------------------------------------
    def call(self, name: str, *args) -> None:
        fn = getattr(self.lib, name)
        rc = fn(C.byref(self.dmesh.struct), C.byref(self.cstruct), C.byref(self.state.struct),
                *args, _stream_ptr())
        _lib.check(rc, name)

    # -- state ---------------------------------------------------------------------------
    def _to_device_order(self, data: Mapping[str, Any]) -> Mapping[str, Any]:
        if self._perm is None:
            return data
        from .reorder import apply_permutation
        return apply_permutation(data, self._perm, self._dims)

    def prepare(self, loaded: Mapping[str, Any]) -> None:
        """Cold-start preparation on the device from loaded theta, rho, qv, u, w."""
        loaded = self._to_device_order(loaded)
        dev = self.dmesh.device
        L = self.dmesh.nVertLevels
        nc = self.dmesh.nCells
        self.state.load(loaded, keys=("u", "w", "scalars", "rt_diabatic_tend"))
        tmp = {}
        for k in ("theta", "rho", "qv"):
            if k in loaded:
                t = torch.as_tensor(_np(loaded[k])[:nc + 1, :L], dtype=torch.float64).to(dev)
                tmp[k] = t.contiguous()
        if "theta" not in tmp or "rho" not in tmp:
            raise MpasConfigError("preparation needs theta and rho")
        qv = tmp.get("qv")
        self.call("mpasg_prepare", C.c_void_p(tmp["theta"].data_ptr()),
                  C.c_void_p(tmp["rho"].data_ptr()),
                  C.c_void_p(qv.data_ptr()) if qv is not None else C.c_void_p(0))
        torch.cuda.current_stream().synchronize()

    def load_boundary(self, state: Mapping[str, Any]) -> None:
        """Load a prepared (complete) step boundary (caller's order)."""
        self.state.load(state, keys=STATE_KEYS + ("rho_edge",), rows=self._rows_in, pending=self._pending_d2h)
        self.state.f["rho_zz"][self.dmesh.nCells].fill_(1.0)

    def prepare_derived(self, state: Mapping[str, Any]) -> None:
        """Load a step boundary and re-derive its coupled diagnostics, solve diagnostics and
        cell winds from its prognostics u, w, theta_m, rho_zz (the reference's treatment of a
        boundary whose prognostics were edited, init_coupled_diagnostics.py:259)."""
        self.load_boundary(state)
        f = self.state.f
        self.call("mpasg_prepare_derived", C.c_void_p(f["theta_m"].data_ptr()), C.c_void_p(f["rho_zz"].data_ptr()))
        torch.cuda.current_stream().synchronize()

    def export_to(self, host: Mapping[str, torch.Tensor]) -> None:
        """Copy the step boundary (caller's order) into the caller's host tensors, one
        field after another on a copy stream of its own.  The copies run while the
        compute stream goes on: a later ``load_boundary`` from the same host tensors waits
        for each field's copy just before it reads that field, so the copies in and out
        of a chain of steps overlap field by field.  Call ``wait_exports`` (or
        synchronise the device) before reading the host tensors."""
        cur = torch.cuda.current_stream()
        if self._d2h_stream is None:
            self._d2h_stream = _copy_stream(self.dmesh.device)
        side = self._d2h_stream
        ex = self.state.export()
        for k, dst in host.items():
            if k not in ex:
                raise MpasConfigError(f"export_to: {k!r} is not a field of the step boundary")
            src = self._export_field(k, ex[k]) if self._perm is not None else ex[k].clone()  # a snapshot
            if tuple(dst.shape) != tuple(src.shape):
                raise MpasConfigError(f"export_to: {k}: shape {tuple(dst.shape)} != {tuple(src.shape)}")
            ready = torch.cuda.Event()
            ready.record(cur)
            side.wait_event(ready)
            with torch.cuda.stream(side):
                dst.copy_(src, non_blocking=True)
            src.record_stream(side)
            done = torch.cuda.Event()
            done.record(side)
            self._pending_d2h[dst.data_ptr()] = done

    def wait_exports(self) -> None:
        """Make the current stream wait for every ``export_to`` copy issued so far."""
        for side in (self._d2h_stream, self._h2d_stream):
            if side is not None:
                torch.cuda.current_stream().wait_stream(side)
        self._pending_d2h.clear()

    def step(self) -> None:
        if self._graph is not None:
            self._graph.replay()
        else:
            self.call("mpasg_step")

    def capture_graph_parts(self) -> None:
        """Capture the two parts of a large step (``mpasg_step_part``) as two CUDA graphs,
        replayed by ``step_host``."""
        torch.cuda.synchronize()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        graphs = []
        for part in (0, 1):
            if part == 1 and not self._has_split_transport():
                graphs.append(None)  # part 1 launches nothing: no graph to capture or replay
                continue
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(s):
                with torch.cuda.graph(g, stream=s):
                    rc = self.lib.mpasg_step_part(C.byref(self.dmesh.struct), C.byref(self.cstruct),
                                                  C.byref(self.state.struct), part, C.c_void_p(s.cuda_stream))
            _lib.check(rc, f"mpasg_step_part {part} (capture)")
            graphs.append(g)
        torch.cuda.current_stream().wait_stream(s)
        self._graph_parts = graphs

    def _has_split_transport(self) -> bool:
        """Whether the second part of a step (the split scalar transport) does any work:
        scalars present, advection on and more than one dynamics substep (one substep is
        the coupled mode, which transports inside the RK stages)."""
        c = self.cstruct
        return c.num_scalars > 0 and not c.scalar_advection_off and c.dynamics_split_steps > 1

    def _step_part(self, part: int) -> None:
        if part == 1 and not self._has_split_transport():
            return
        if self._graph_parts is not None:
            self._graph_parts[part].replay()
        else:
            self.call("mpasg_step_part", part)

    def step_host(self, host: Mapping[str, torch.Tensor]) -> None:
        """Advance a step boundary held in (pinned) host tensors by one large step, in
        place: ``load_boundary(host)``, the first part of the step, ``export_to`` of every
        field that is final by then (all but the scalars), which copies out while the
        second part (the scalar transport) runs, then ``export_to`` of the scalars.  Call ``wait_exports`` before reading ``host``."""
        self.load_boundary(host)
        late = {k: v for k, v in host.items() if k in LATE_KEYS}
        early = {k: v for k, v in host.items() if k not in LATE_KEYS}
        self._step_part(0)
        self.export_to(early)
        self._step_part(1)
        self.export_to(late)

    def run_host(self, host: Mapping[str, torch.Tensor], nsteps: int) -> None:
        """Advance a step boundary held in pinned host tensors by ``nsteps`` large steps,
        in place, copying every step's boundary in from ``host`` and its result back out to
        ``host`` (the same fields as ``step_host``).  The copies are pipelined on two copy
        streams: each field of a step's result is copied out as soon as it is final (most
        of them while the scalar transport runs), and copied back in, for the next step,
        into a device staging buffer as soon as its copy out has finished; a step starts
        once all of its inputs are staged.  Returns with the current stream ordered after
        every copy (``host`` is complete once the current stream reaches that point)."""
        from .device import ALIASES, ENTITY, FIELD_KIND
        if self._graph_parts is None:
            self.capture_graph_parts()
        dev = self.dmesh.device
        cur = torch.cuda.current_stream(dev)
        if self._d2h_stream is None:
            self._d2h_stream = _copy_stream(dev)
        if self._h2d_stream is None:
            self._h2d_stream = _copy_stream(dev)
        down, up = self._d2h_stream, self._h2d_stream
        # the copy streams start after everything issued so far (an earlier call's copies
        # out into these host tensors, loads, steps)
        up.wait_stream(cur)
        down.wait_stream(cur)
        names = {k: ALIASES.get(k, k) for k in host}
        for k, n in names.items():
            if n not in self.state.f or tuple(host[k].shape) != tuple(self.state.f[n].shape):
                raise MpasConfigError(f"run_host: {k!r} is not a field of the step boundary with its shape")
        staging = {k: torch.empty_like(self.state.f[n]) for k, n in names.items()}
        rows = {k: (self._rows_in[ENTITY[FIELD_KIND[n]]] if self._perm is not None else None) for k, n in names.items()}
        ready = {}
        for k in host:  # the first step's inputs
            ev = self._pending_d2h.pop(host[k].data_ptr(), None)
            if ev is not None:
                up.wait_event(ev)
            with torch.cuda.stream(up):
                staging[k].copy_(host[k], non_blocking=True)
            ready[k] = torch.cuda.Event()
            ready[k].record(up)
        static = [k for k in host if k in STATIC_KEYS]
        late = [k for k in host if k in LATE_KEYS]
        early = [k for k in host if k not in LATE_KEYS and k not in STATIC_KEYS]
        for step in range(int(nsteps)):
            for k, n in names.items():  # load the staged inputs into the state
                cur.wait_event(ready[k])
                if rows[k] is not None:
                    self.state.gather_rows(staging[k], rows[k], out=self.state.f[n])
                else:
                    self.state.f[n].copy_(staging[k])
            self.state.f["rho_zz"][self.dmesh.nCells].fill_(1.0)
            last = step == int(nsteps) - 1
            # fields the step never writes are final once loaded; the others after the
            # part of the step that writes them last
            for part, keys in ((None, static), (0, early), (1, late)):
                if part is not None:
                    self._step_part(part)
                final = torch.cuda.Event()
                final.record(cur)
                down.wait_event(final)
                for k in keys:
                    with torch.cuda.stream(down):
                        src = self._export_field(k, self.state.f[names[k]]) if self._perm is not None \
                            else self.state.f[names[k]]
                        host[k].copy_(src, non_blocking=True)
                    if last:
                        continue
                    done = torch.cuda.Event()
                    done.record(down)
                    up.wait_event(done)  # the next step's input is this step's output
                    with torch.cuda.stream(up):
                        staging[k].copy_(host[k], non_blocking=True)
                    ready[k] = torch.cuda.Event()
                    ready[k].record(up)
        for k in staging:
            staging[k].record_stream(up)
        # the state is not touched again before the last copies out have read it
        cur.wait_stream(down)
        cur.wait_stream(up)

    def capture_graph(self) -> None:
        """Capture one large step as a CUDA graph (replayed by ``step``)."""
        torch.cuda.synchronize()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            # warm-up outside capture is the caller's job; capture the launch sequence
            with torch.cuda.graph(g, stream=s):
                fn = self.lib.mpasg_step
                rc = fn(C.byref(self.dmesh.struct), C.byref(self.cstruct), C.byref(self.state.struct),
                        C.c_void_p(s.cuda_stream))
        torch.cuda.current_stream().wait_stream(s)
        _lib.check(rc, "mpasg_step (capture)")
        self._graph = g

    def autotune(self) -> dict:
        """Pick the tile shapes of the tuned kernels on this mesh and state
        (``mpasg_autotune``); returns the measured times per candidate (ms)."""
        times = (C.c_float * 3)()
        torch.cuda.synchronize()
        rc = self.lib.mpasg_autotune(C.byref(self.dmesh.struct), C.byref(self.cstruct), C.byref(self.state.struct),
                                     times, _stream_ptr())
        _lib.check(rc, "mpasg_autotune")
        self._graph = self._graph_parts = None  # captured graphs hold the old tile
        return {"tend_u_levels_per_thread": int(self.cstruct.tile_tend_u),
                "tend_u_ms": {1: times[0], 2: times[1], 4: times[2]}}

    def check_finite(self) -> int:
        self.call("mpasg_check_finite")
        return int(self.state.status[0].item())

    def export(self, clone: bool = True) -> dict[str, torch.Tensor]:
        """The step boundary in the caller's order (``clone=False``: views of the device
        fields where no reordering is needed)."""
        if self._perm is None:
            ex = self.state.export()
            return {k: v.clone() for k, v in ex.items()} if clone else dict(ex)
        return {k: self._export_field(k, v) for k, v in self.state.export().items()}

    def _export_field(self, key: str, v: torch.Tensor) -> torch.Tensor:
        """One device field gathered into the caller's row order."""
        from .device import ALIASES, ENTITY, FIELD_KIND
        return self.state.gather_rows(v, self._rows_out[ENTITY[FIELD_KIND[ALIASES.get(key, key)]]])


def _is_prepared(state: Mapping[str, Any]) -> bool:
    return all(k in state for k in ("theta_m", "rho_zz", "rtheta_p", "exner", "pv_edge", "v"))


def _merge(base: Mapping[str, Any], out: Mapping[str, torch.Tensor]) -> dict:
    res = dict(base)
    res.pop(MARKER, None)
    res.update(out)
    return res


def _start(model: "Model", state: Mapping[str, Any], merged: Mapping[str, Any], complete: bool) -> None:
    """Bring the model to the start boundary as the reference's _prepare_timestep_state
    does (atmosphere_model.py:782-898): a complete bound boundary continues as it is; any
    other state is prepared, from theta_m and rho_zz where it has both (a boundary whose
    prognostics were edited), else from the loaded theta, rho and qv."""
    if complete:
        model.load_boundary(state)
    elif "theta_m" in merged and "rho_zz" in merged and _is_prepared(state):
        model.prepare_derived(state)
    else:
        model.prepare(merged)


def _check_boundary(state: Mapping[str, Any], mesh: Mapping[str, Any] | None, cfg: Mapping[str, Any],
                    dt: float) -> bool:
    """The continuation checks of a start state (atmosphere_model.py:829-838): a marked
    state continues only with its own mesh, configuration and time step, and only its
    prognostics may have been edited.  Returns whether it is a complete boundary."""
    require_boundary_continuation_identity(state, mesh=mesh, config=cfg, dt=dt)
    complete = has_complete_step_boundary(state)
    if not complete:
        require_unedited_boundary_support(state)
    return complete


def run_simulation(initial_state: Mapping[str, Any], mesh: Mapping[str, Any] | None = None,
                   config: Mapping[str, Any] | None = None, dt: float | None = None, nsteps: int = 1,
                   device: str | torch.device = "cuda", on_step: Callable | None = None,
                   differentiable: bool = False, checkpoint_timesteps: bool | None = None,
                   checkpoint_use_reentrant: bool = False, checkpoint_materialize_final: bool = True,
                   on_phase: Callable | None = None, on_initial: Callable | None = None,
                   use_cuda_graph: bool = True) -> dict:
    """Forecast ``nsteps`` large steps on the GPU (reference: atmosphere_model.py:1474).

    ``initial_state`` is either a loaded raw state (prepared here, on the device) or a
    complete step boundary returned by a previous call.  Returns the final boundary with
    the reference's keys; tensors stay on the CUDA device.  With ``differentiable=True``:
    ``initial_state["scalars"]`` requiring grad, the returned ``scalars`` carry the
    hand-written adjoint of the scalar transport into autograd (passive scalars, explicit
    split transport); the loaded ``u``, ``w``, ``theta`` or ``rho`` requiring grad, the
    returned fields carry the hand-written reverse mode of the dynamics (per-step
    checkpoints, or every step's tape with ``checkpoint_timesteps=False``, whose forward
    advances the dynamics only, so its result has no scalars or reconstructed winds); other inputs
    requiring grad are rejected before any device work.
    """
    return _simulate(initial_state, mesh, config, dt, nsteps, device, on_step, differentiable, on_phase, on_initial,
                     use_cuda_graph, bound=True, checkpoint_timesteps=checkpoint_timesteps)


def _simulate(initial_state, mesh, config, dt, nsteps, device, on_step, differentiable, on_phase, on_initial,
              use_cuda_graph, bound: bool, checkpoint_timesteps: bool | None = None) -> dict:
    """run_simulation's body; ``bound`` False (atm_srk3) continues from the given prepared
    state as it is and returns an unbound result."""
    reject_unsupported_request(initial_state, mesh, config)
    require_finite_inputs(initial_state)
    if int(nsteps) != nsteps or nsteps < 0:
        raise MpasConfigError("nsteps must be a non-negative integer")
    if differentiable and _grad_keys(initial_state, mesh) and nsteps > 0:
        return _run_differentiable(initial_state, mesh, config, dt, int(nsteps), device, on_step, on_phase,
                                   on_initial, {"checkpoint_timesteps": checkpoint_timesteps})
    # a boundary is bound to the mesh the caller passed (none when the state is its own mesh)
    boundary_mesh = dict(mesh) if mesh is not None else None
    mesh = mesh if mesh is not None else initial_state
    merged = dict(mesh)
    merged.update(initial_state)
    cfg = resolved_config(config)
    dt = float(cfg["config_dt"] if dt is None else dt)
    if nsteps == 0:
        return dict(initial_state)
    if _flag(cfg, "config_mesh_reordering_rcm") and not merged.get("_rcm_applied", False):
        # the reference reorders state and mesh and updates the caller's mesh in place
        # (atmosphere_model.py:810-827); results come back in the RCM order
        from .reorder import apply_rcm_reordering
        initial_state, new_mesh = apply_rcm_reordering(initial_state, mesh)
        if isinstance(mesh, dict):
            mesh.clear()
            mesh.update(new_mesh)
        else:
            mesh = new_mesh
        merged = dict(mesh)
        merged.update(initial_state)
    complete = _check_boundary(initial_state, boundary_mesh, cfg, dt) if bound else True
    ns = _int(merged.get("num_scalars", _np(merged["scalars"]).shape[-1]))
    model = Model(merged, cfg, dt, num_scalars=ns, device=device)
    _start(model, initial_state, merged, complete)
    if on_initial is not None:
        on_initial(_merge(initial_state, model.export()))
    if on_phase is not None:
        on_phase("forecast_integration_begin")
    if use_cuda_graph and nsteps > 1:
        model.step()
        model.capture_graph()
        first = 1
        if on_step is not None:
            on_step(1, _merge(initial_state, model.export()))
    else:
        first = 0
    for i in range(first, int(nsteps)):
        model.step()
        if on_step is not None:
            on_step(i + 1, _merge(initial_state, model.export()))
    if on_phase is not None:
        on_phase("forecast_integration_end")
    bad = model.check_finite()
    if bad:
        raise MpasNumericalError(f"forecast result contains {bad} nonfinite values")
    out = _merge(initial_state, model.export())
    if bound:
        # the returned boundary continues a later call as it is (atmosphere_model.py:2024-2032)
        mark_complete_step_boundary(out, mesh=boundary_mesh, config=cfg, dt=dt)
    return out


def _scalar_derivative_forward(state: Mapping[str, Any], mesh: Mapping[str, Any] | None, kwargs: dict):
    """Forward run for run_simulation.vjp / .jvp with each step's transport inputs taped."""
    from .tracer_adjoint import ScalarTape, check_supported
    unknown = set(kwargs) - {"config", "dt", "nsteps", "device", "differentiable", "checkpoint_timesteps",
                             "checkpoint_use_reentrant", "checkpoint_materialize_final"}
    if unknown:
        raise MpasConfigError(f"unsupported keyword arguments for the derivative runs: {sorted(unknown)}")
    mesh = mesh if mesh is not None else state
    merged = dict(mesh)
    merged.update(state)
    cfg = resolved_config(kwargs.get("config"))
    dt = float(cfg["config_dt"] if kwargs.get("dt") is None else kwargs["dt"])
    nsteps = int(kwargs.get("nsteps", 1))
    ns = _int(merged.get("num_scalars", _np(merged["scalars"]).shape[-1]))
    # the Model's defaults: every scalar is a moist species unless moist_end says otherwise
    ms, me = _int(merged.get("moist_start", 1)), _int(merged.get("moist_end", ns))
    check_supported(cfg, ms, me)
    complete = _check_boundary(state, None if mesh is state else mesh, cfg, dt)
    model = Model(merged, cfg, dt, num_scalars=ns, device=kwargs.get("device", "cuda"))
    _start(model, state, merged, complete)
    tape = ScalarTape(model)
    for i in range(nsteps):
        tape.step(model)
        if i == 0 and nsteps > 1 and not tape.coupled:
            model.capture_graph()  # later steps replay the step graph (bitwise the eager step)
    bad = model.check_finite()
    if bad:
        raise MpasNumericalError(f"forecast result contains {bad} nonfinite values")
    return model, tape, _merge(state, model.export())


DYNAMICS_GRAD_KEYS = ("u", "w", "theta", "rho")


def _grad_keys(state: Mapping[str, Any], mesh: Mapping[str, Any] | None) -> list[str]:
    """The inputs that require gradients: ``scalars`` (the hand-written adjoint of the
    scalar transport) or any of the loaded ``u``, ``w``, ``theta``, ``rho`` (that of the
    dynamics), not both; checked before any device work."""
    keys = sorted({k for d in (state, mesh or {}) for k, v in d.items()
                   if isinstance(v, torch.Tensor) and v.requires_grad})
    other = [k for k in keys if k != "scalars" and k not in DYNAMICS_GRAD_KEYS]
    mesh_keys = [k for k in keys if mesh is not None and k in mesh and k not in state]
    if other or mesh_keys or ("scalars" in keys and len(keys) > 1):
        raise MpasUnsupportedCapabilityError(
            "differentiable runs on the GB300 path carry gradients for 'scalars' (hand-written adjoint of the "
            "scalar transport) or for the loaded u, w, theta, rho (that of the dynamics), not both; inputs "
            f"requiring grad: {keys}")
    return keys


class _ScalarsThroughSteps(torch.autograd.Function):
    """The end scalars of a taped forward as a function of the start scalars: forward
    returns the already computed result, backward runs the hand-written transposed
    transport of every taped step (``mpasg_transport_vjp``)."""

    @staticmethod
    def forward(ctx, scalars_in, scalars_end, model, tape):  # noqa: D401
        ctx.model, ctx.tape = model, tape
        ctx.in_rows, ctx.in_device = scalars_in.shape[0], scalars_in.device
        return scalars_end.detach().clone()

    @staticmethod
    def backward(ctx, g_end):
        from .tracer_adjoint import scalars_vjp
        g0 = scalars_vjp(ctx.model, ctx.tape, g_end.detach())[:ctx.in_rows]
        return g0.to(ctx.in_device), None, None, None


class _DynamicsThroughSteps(torch.autograd.Function):
    """The final state of a run as a function of the loaded u, w, theta, rho: forward
    runs the forward phase of a ``dyn_adjoint.VjpRun`` (the steps with their checkpoints)
    and returns every floating field of the final state; backward hands the cotangents of
    the carried fields (and ``rho_edge``) to the run's reverse phase (the hand-written
    reverse mode) and returns the inputs' gradients.  A nonzero cotangent of any other
    output (the scalars, the reconstructed winds, ...) is refused: no derivative through it
    is built, and dropping it would give a wrong gradient."""

    @staticmethod
    def forward(ctx, run, names, keys, *inputs):  # noqa: D401
        ctx.set_materialize_grads(False)
        ctx.run, ctx.names, ctx.keys = run, names, keys
        ctx.in_meta = [(x.shape[0], x.device) for x in inputs]
        final = run.final
        return tuple(final[k] for k in names)

    @staticmethod
    def backward(ctx, *g_out):
        from .dyn_adjoint import DIFFERENTIABLE_OUT
        g = {}
        for k, v in zip(ctx.names, g_out):
            if v is None:
                continue
            if k not in DIFFERENTIABLE_OUT:
                if bool(torch.any(v != 0)):
                    raise MpasUnsupportedCapabilityError(f"the derivative through output {k!r} is not built")
                continue
            g[k] = v.detach()
        grads = ctx.run.reverse(g)
        res = [grads[k][:rows].to(dev) for k, (rows, dev) in zip(ctx.keys, ctx.in_meta)]
        return (None, None, None, *res)


def _run_differentiable_dynamics(state, mesh, config, dt, nsteps, device, keys, kwargs) -> dict:
    """run_simulation(differentiable=True) with the loaded u, w, theta or rho requiring grad:
    the forward phase of the dynamics' reverse mode (per-step checkpoints, or the modes of
    ``checkpoint_timesteps`` / the configuration's ``gradient_checkpointing`` as for
    run_simulation.vjp), its final state attached to the autograd graph through
    ``_DynamicsThroughSteps``."""
    from .dyn_adjoint import DynamicsAdjoint, VjpRun, check_request
    if _is_prepared(state):
        raise MpasUnsupportedCapabilityError(
            "dynamics derivatives start from a loaded (unprepared) state: track u, w, theta or rho")
    mesh = mesh if mesh is not None else state
    plain = {k: (v.detach() if isinstance(v, torch.Tensor) else v) for k, v in state.items()}
    merged = dict(mesh)
    merged.update(plain)
    cfg = resolved_config(config)
    dt = float(cfg["config_dt"] if dt is None else dt)
    ns = _int(merged.get("num_scalars", _np(merged["scalars"]).shape[-1]))
    check_request(cfg, merged, ns, allow_mixed=True)
    model = Model(merged, cfg, dt, num_scalars=ns, device=device)
    run = VjpRun(model, merged, nsteps, DynamicsAdjoint(model), checkpoint=_checkpoint_mode(config, kwargs))
    run.final = run.forward()
    out = _merge(plain, run.final)
    # with every step's tape kept (checkpoint_timesteps=False) the forward advances the
    # dynamics only: the scalars and the reconstructed winds are not part of the result
    # (not the loaded ones passed through)
    for k in ("scalars", "uReconstructX", "uReconstructY", "uReconstructZ", "uReconstructZonal",
              "uReconstructMeridional", "ur_cell", "vr_cell"):
        if k not in run.final:
            out.pop(k, None)
    names = tuple(k for k, v in run.final.items()
                  if k not in STATIC_KEYS and isinstance(v, torch.Tensor) and torch.is_floating_point(v))
    attached = _DynamicsThroughSteps.apply(run, names, tuple(keys), *[state[k] for k in keys])
    out.update(dict(zip(names, attached)))
    return out


def _checkpoint_mode(config, kwargs) -> str:
    """checkpoint_timesteps=False keeps every step's tape (no recomputation), as the
    reference keeps the whole graph without its per-step checkpoint; gradient_checkpointing
    in the configuration (the reference's nested recomputation inside the step) recomputes
    every dynamics substep from its step's checkpoint and keeps sqrt(nsteps) step checkpoints
    (atmosphere_model.py:120-154); otherwise one checkpoint per step."""
    if kwargs.get("checkpoint_timesteps") is False:
        return "none"
    if "gradient_checkpointing" in (config or {}) and _flag(dict(config), "gradient_checkpointing"):
        return "sqrt"
    return "step"


def _run_differentiable(state, mesh, config, dt, nsteps, device, on_step, on_phase, on_initial,
                        kwargs=None) -> dict:
    """run_simulation(differentiable=True) with inputs requiring grad.  ``scalars``: the
    taped forward, and the end scalars attached to the autograd graph through
    ``_ScalarsThroughSteps`` (passive scalars, explicit split transport); the loaded u, w,
    theta, rho: ``_run_differentiable_dynamics``."""
    if on_step is not None or on_initial is not None:
        raise MpasUnsupportedCapabilityError("on_step / on_initial are not available in differentiable runs")
    keys = _grad_keys(state, mesh)
    if "scalars" not in keys:
        if on_phase is not None:
            on_phase("forecast_integration_begin")
        out = _run_differentiable_dynamics(state, mesh, config, dt, nsteps, device, keys, kwargs or {})
        if on_phase is not None:
            on_phase("forecast_integration_end")
        return out
    plain = {k: (v.detach() if isinstance(v, torch.Tensor) else v) for k, v in state.items()}
    if on_phase is not None:
        on_phase("forecast_integration_begin")
    model, tape, out = _scalar_derivative_forward(plain, mesh, {"config": config, "dt": dt, "nsteps": nsteps,
                                                                "device": device})
    if on_phase is not None:
        on_phase("forecast_integration_end")
    out = dict(out)
    out["scalars"] = _ScalarsThroughSteps.apply(state["scalars"], out["scalars"], model, tape)
    return out


def _objective_loss(objective: Callable, out: Mapping[str, Any]) -> torch.Tensor:
    loss = objective(out)
    if not isinstance(loss, torch.Tensor):
        raise TypeError(f"objective must return a tensor, got {type(loss).__name__}")
    if loss.ndim != 0:
        raise MpasConfigError("objective must return a scalar tensor")
    return loss


def _dynamics_vjp(state: Mapping[str, Any], mesh: Mapping[str, Any] | None, objective: Callable,
                  keys: tuple, kwargs: dict) -> dict:
    """run_simulation.vjp with respect to the loaded u, w, theta, rho: the hand-written
    reverse mode of the dynamics (dyn_adjoint.py, ``mpasg_step_vjp``)."""
    from .dyn_adjoint import DIFFERENTIABLE_OUT, DynamicsAdjoint, check_request, run_vjp
    unknown = set(kwargs) - {"config", "dt", "nsteps", "device", "differentiable", "checkpoint_timesteps",
                             "checkpoint_use_reentrant", "checkpoint_materialize_final"}
    if unknown:
        raise MpasConfigError(f"unsupported keyword arguments for the derivative runs: {sorted(unknown)}")
    for k in keys:
        if k not in state or not hasattr(state[k], "shape"):
            raise KeyError(f"Tracked VJP key '{k}' is missing from state")
    if _is_prepared(state):
        raise MpasUnsupportedCapabilityError(
            "dynamics derivatives start from a loaded (unprepared) state: track u, w, theta or rho")
    mesh = mesh if mesh is not None else state
    merged = dict(mesh)
    merged.update(state)
    cfg = resolved_config(kwargs.get("config"))
    dt = float(cfg["config_dt"] if kwargs.get("dt") is None else kwargs["dt"])
    nsteps = int(kwargs.get("nsteps", 1))
    ns = _int(merged.get("num_scalars", _np(merged["scalars"]).shape[-1]))
    check_request(cfg, merged, ns, allow_mixed=True)
    model = Model(merged, cfg, dt, num_scalars=ns, device=kwargs.get("device", "cuda"))
    adj = DynamicsAdjoint(model)

    def cotangents(final: dict) -> dict:
        out = _merge(state, final)
        leaves = {k: out[k].detach().clone().requires_grad_(True) for k in DIFFERENTIABLE_OUT
                  if isinstance(out.get(k), torch.Tensor)}
        # every other output the step computes is a leaf too: a derivative through it is
        # refused (the base state and the diabatic forcing are constants of the run)
        others = {k: v.detach().clone().requires_grad_(True) for k, v in final.items()
                  if k not in leaves and k not in STATIC_KEYS and isinstance(v, torch.Tensor)
                  and torch.is_floating_point(v)}
        loss = _objective_loss(objective, {**out, **leaves, **others})
        names = list(leaves) + list(others)
        grads = torch.autograd.grad(loss, [leaves.get(k, others.get(k)) for k in names], allow_unused=True)
        res = {}
        for k, g in zip(names, grads):
            if g is None:
                continue
            if k in others:
                if bool(torch.any(g != 0)):
                    raise MpasUnsupportedCapabilityError(f"the objective's derivative through {k!r} is not built")
                continue
            res[k] = g.detach()
        return res

    grads, _ = run_vjp(model, merged, nsteps, cotangents, adj,
                       checkpoint=_checkpoint_mode(kwargs.get("config"), kwargs))
    res = {}
    for k in keys:
        ref = state[k]
        g = grads[k][:ref.shape[0]]
        res[k] = g if isinstance(ref, torch.Tensor) and ref.device == g.device else \
            (g.to(ref.device) if isinstance(ref, torch.Tensor) else g.cpu())
    return res


def run_simulation_vjp(state: Mapping[str, Any], mesh: Mapping[str, Any], objective: Callable,
                       track_keys=None, **kwargs) -> dict:
    """Adjoint of ``run_simulation`` (the reference's ``run_simulation.vjp``,
    atmosphere_model.py:2101): d objective(out) / d state[key] through ``nsteps`` steps.

    * ``track_keys`` within ``("u", "w", "theta", "rho")``: the loaded wind, vertical wind,
      potential temperature and density, through the preparation and the dynamics (the
      hand-written reverse mode of dyn_adjoint.py: dry, flat or terrain-following levels,
      float64 or the mixed
      form, every mixing and damping option; the objective may read the step boundary's
      carried fields);
    * ``track_keys=("scalars",)``: the transported scalars, by the hand-written transposed
      transport (``mpasg_transport_vjp``; passive scalars, explicit split transport)."""
    from .tracer_adjoint import scalars_vjp
    reject_unsupported_request(state, mesh, kwargs.get("config"))
    keys = tuple(track_keys) if track_keys is not None else None
    if keys and all(k in ("u", "w", "theta", "rho") for k in keys):
        return _dynamics_vjp(state, mesh, objective, keys, dict(kwargs))
    if keys != ("scalars",):
        raise MpasUnsupportedCapabilityError(
            "run_simulation.vjp on the GB300 path differentiates with respect to 'scalars', or to any of "
            f"'u', 'w', 'theta', 'rho' (not both kinds at once); got {keys}")
    if "scalars" not in state or not hasattr(state["scalars"], "shape"):
        raise KeyError("Tracked VJP key 'scalars' is missing from state")
    model, tape, out = _scalar_derivative_forward(state, mesh, dict(kwargs))
    leaf = out["scalars"].detach().clone().requires_grad_(True)
    out = dict(out)
    out["scalars"] = leaf
    loss = objective(out)
    if not isinstance(loss, torch.Tensor):
        raise TypeError(f"objective must return a tensor, got {type(loss).__name__}")
    if loss.ndim != 0:
        raise MpasConfigError("objective must return a scalar tensor")
    (g_end,) = torch.autograd.grad(loss, [leaf], allow_unused=True)
    if g_end is None:
        return {}
    g0 = scalars_vjp(model, tape, g_end.detach())
    ref = state["scalars"]
    g0 = g0[:ref.shape[0]]
    return {"scalars": g0 if isinstance(ref, torch.Tensor) and ref.device == g0.device else
            (g0.to(ref.device) if isinstance(ref, torch.Tensor) else g0.cpu())}


def _check_perturbation(state: Mapping[str, Any], perturbation: Mapping[str, Any]) -> None:
    """The reference's checks of a tangent (atmosphere_model.py:2065-2090)."""
    for key, tangent in perturbation.items():
        if not isinstance(tangent, torch.Tensor):
            raise TypeError(f"Perturbation '{key}' must be a tensor, got {type(tangent).__name__}")
        if key not in state:
            raise KeyError(f"Perturbation '{key}' is missing from state")
        ref = state[key]
        if not isinstance(ref, torch.Tensor):
            raise TypeError(f"State entry '{key}' is not a tensor and cannot receive a tangent")
        if tangent.shape != ref.shape:
            raise MpasConfigError(f"Perturbation '{key}' has shape {tuple(tangent.shape)}; expected {tuple(ref.shape)}")
        if tangent.dtype != ref.dtype:
            raise MpasConfigError(f"Perturbation '{key}' has dtype {tangent.dtype}; expected {ref.dtype}")
        if tangent.device != ref.device:
            raise MpasConfigError(f"Perturbation '{key}' is on {tangent.device}; expected {ref.device}")


def _dynamics_jvp(state: Mapping[str, Any], mesh: Mapping[str, Any] | None, perturbation: Mapping[str, Any],
                  kwargs: dict) -> dict:
    """run_simulation.jvp along the loaded u, w, theta, rho: the hand-written forward mode of
    the dynamics (dyn_adjoint.py, ``mpasg_step_jvp``)."""
    from .dyn_adjoint import DynamicsTangent, check_request, run_jvp
    unknown = set(kwargs) - {"config", "dt", "nsteps", "device", "differentiable", "checkpoint_timesteps",
                             "checkpoint_use_reentrant", "checkpoint_materialize_final"}
    if unknown:
        raise MpasConfigError(f"unsupported keyword arguments for the derivative runs: {sorted(unknown)}")
    if _is_prepared(state):
        raise MpasUnsupportedCapabilityError(
            "dynamics derivatives start from a loaded (unprepared) state: perturb u, w, theta or rho")
    mesh = mesh if mesh is not None else state
    merged = dict(mesh)
    merged.update(state)
    cfg = resolved_config(kwargs.get("config"))
    dt = float(cfg["config_dt"] if kwargs.get("dt") is None else kwargs["dt"])
    nsteps = int(kwargs.get("nsteps", 1))
    ns = _int(merged.get("num_scalars", _np(merged["scalars"]).shape[-1]))
    check_request(cfg, merged, ns)
    model = Model(merged, cfg, dt, num_scalars=ns, device=kwargs.get("device", "cuda"))
    tangents = run_jvp(model, merged, nsteps, perturbation, DynamicsTangent(model))
    dev = next(iter(perturbation.values())).device
    return {k: v.to(dev) for k, v in tangents.items()}


def run_simulation_jvp(state: Mapping[str, Any], mesh: Mapping[str, Any], perturbation: Mapping[str, Any],
                       **kwargs) -> dict:
    """Tangent-linear ``run_simulation`` (the reference's ``run_simulation.jvp``,
    atmosphere_model.py:2041).

    * a perturbation of any of ``u``, ``w``, ``theta``, ``rho`` (the loaded primitives):
      tangents of the final dynamics fields (the carried fields and ``rho_edge``) through the
      preparation and the dynamics (the hand-written forward mode of dyn_adjoint.py: dry,
      flat or terrain-following levels, float64).  The scalars' tangent along the winds is not formed;
    * ``perturbation["scalars"]``: the tangent of the end scalars, replayed through each
      step's recorded transport.  Outputs that do not depend on the scalars get no tangent,
      as in the reference."""
    from .tracer_adjoint import scalars_jvp
    reject_unsupported_request(state, mesh, kwargs.get("config"))
    _check_perturbation(state, perturbation)
    if perturbation and set(perturbation) <= {"u", "w", "theta", "rho"}:
        return _dynamics_jvp(state, mesh, perturbation, dict(kwargs))
    if set(perturbation) != {"scalars"}:
        raise MpasUnsupportedCapabilityError(
            "run_simulation.jvp on the GB300 path takes a 'scalars' perturbation, or one of any of 'u', 'w', "
            f"'theta', 'rho' (not both kinds at once); got {sorted(perturbation)}")
    v = perturbation["scalars"]
    if not isinstance(v, torch.Tensor):
        raise TypeError(f"Perturbation 'scalars' must be a tensor, got {type(v).__name__}")
    ref = state["scalars"]
    if tuple(v.shape) != tuple(ref.shape):
        raise MpasConfigError(f"Perturbation 'scalars' has shape {tuple(v.shape)}; expected {tuple(ref.shape)}")
    model, tape, _ = _scalar_derivative_forward(state, mesh, dict(kwargs))
    dev = model.dmesh.device
    full = torch.zeros(model.state.f["scalars"].shape, dtype=torch.float64, device=dev)
    full[:v.shape[0]] = v.to(device=dev, dtype=torch.float64)
    t = scalars_jvp(model, tape, full)[:v.shape[0]]
    return {"scalars": t.to(v.device)}


run_simulation.vjp = run_simulation_vjp  # type: ignore[attr-defined]
run_simulation.jvp = run_simulation_jvp  # type: ignore[attr-defined]


def run_timestep(state: Mapping[str, Any], mesh: Mapping[str, Any] | None = None,
                 config: Mapping[str, Any] | None = None, dt: float | None = None,
                 device: str | torch.device = "cuda", differentiable: bool = False) -> dict:
    """One large step (reference: atmosphere_model.py:900)."""
    return run_simulation(state, mesh, config, dt, 1, device, differentiable=differentiable,
                          use_cuda_graph=False)


def atm_srk3(state: Mapping[str, Any], mesh: Mapping[str, Any], config: Mapping[str, Any], dt: float,
             strict: bool = True, differentiable: bool = False) -> dict:
    """One split-explicit RK3 step on a prepared boundary (dynamics/time_integration.py:4897)."""
    if not _is_prepared(state):
        raise MpasConfigError("atm_srk3 needs a prepared step boundary")
    return _simulate(state, mesh, config, dt, 1, "cuda", None, differentiable, None, None, False, bound=False)
