"""Binding of a returned step boundary to its values and continuation identity
(reference: mpas_pytorch/state.py:66-264).

``run_simulation`` marks the boundary it returns.  A later call that gets the same boundary
back continues from it as it is; one whose prognostics (u, w, rho_zz, theta_m, scalars) were
edited re-derives the coupled diagnostics from them; one whose diagnostics or support
inputs were edited, or that continues on another mesh, configuration or time step, is
rejected.  The marker lives under the reference's key with the reference's binding tag.

The reference binds every tensor by a host copy of its bytes.  Here a tensor on a CUDA
device is bound by a 128-bit digest of its bytes computed on the device
(``mpasg_digest``), and a host array by the same digest computed with numpy, so a boundary
keeps its binding through a clone or a move between host and device, and an in-place
edit of any value changes the digest (unless two mixed words collide, about 2^-64 each).
"""

from __future__ import annotations

import json
from typing import Any, Mapping

import numpy as np
import torch

from .errors import MpasConfigError
from .netcdf_io import continuation_configuration_digest, mesh_digest

BOUNDARY_PROGNOSTICS = ("u", "w", "rho_zz", "theta_m", "scalars")  # state.py:66
PRIMARY_ALIASES = {"t": "theta_m"}                                   # state.py:67
MARKER = "_restart_skip_rederivation"                                # state.py:68
BINDING = "mpas-boundary-bytes.v1"                                   # state.py:69
_KEPT_PRIVATE = ("_edge_ordering_mismatch", "_mesh_connectivity_preferred")

_M64 = (1 << 64) - 1
_SEED = 0x9E3779B97F4A7C15
_LANE_B = 0x5851F42D4C957F2D


def _smix(x: np.ndarray) -> np.ndarray:
    """The SplitMix64 output function on uint64 words (wrapping arithmetic)."""
    x = x ^ (x >> np.uint64(30))
    x = x * np.uint64(0xBF58476D1CE4E5B9)
    x = x ^ (x >> np.uint64(27))
    x = x * np.uint64(0x94D049BB133111EB)
    return x ^ (x >> np.uint64(31))


def _smix_int(x: int) -> int:
    x &= _M64
    x ^= x >> 30
    x = (x * 0xBF58476D1CE4E5B9) & _M64
    x ^= x >> 27
    x = (x * 0x94D049BB133111EB) & _M64
    return x ^ (x >> 31)


def _lanes_host(raw: np.ndarray) -> tuple[int, int]:
    """The digest lanes (A, B) of a host byte array (the device kernel's restatement)."""
    nb = raw.size
    if nb == 0:
        return 0, 0
    padded = np.zeros(((nb + 7) // 8) * 8, dtype=np.uint8)
    padded[:nb] = raw
    w = padded.view("<u8")
    with np.errstate(over="ignore"):
        idx = np.arange(w.size, dtype=np.uint64) + np.uint64(_SEED)
        h = _smix(w ^ _smix(idx))
        a = int(h.sum(dtype=np.uint64))
        b = int(_smix(h ^ np.uint64(_LANE_B)).sum(dtype=np.uint64))
    return a, b


def _finish(a: int, b: int, nbytes: int) -> str:
    return f"{_smix_int(a ^ nbytes):016x}{_smix_int(b + nbytes):016x}"


def _device_lanes(t: torch.Tensor, out: torch.Tensor, slot: int) -> None:
    from ._lib import check, load
    if t.data_ptr() % 8:
        t = t.clone()
    rc = load().mpasg_digest(t.data_ptr(), t.numel() * t.element_size(), out[slot].data_ptr(),
                             torch.cuda.current_stream(t.device).cuda_stream)
    check(rc, "mpasg_digest")


def _snapshot(state: Mapping[str, Any], support_only: bool = False) -> dict[str, tuple]:
    """(dtype, shape, digest) of every tensor / array and (``"scalar"``, (), JSON) of every
    number or string of ``state`` (private keys skipped, as state.py:85-141 does).  One
    digest per distinct view within a call; CUDA tensors are digested on their device with
    one copy of all their lanes to the host at the end."""
    snap: dict[str, tuple] = {}
    ref_of: dict[tuple, Any] = {}           # view identity -> digest or (device, slot)
    on_dev: dict[torch.device, list[torch.Tensor]] = {}
    for key, value in state.items():
        if key.startswith("_") and key not in _KEPT_PRIVATE:
            continue
        if support_only and (key in BOUNDARY_PROGNOSTICS or key in PRIMARY_ALIASES):
            continue
        if isinstance(value, (bool, int, float, str, np.generic)):
            item = value.item() if isinstance(value, np.generic) else value
            snap[key] = ("scalar", (), json.dumps(item, sort_keys=True, default=str))
            continue
        if isinstance(value, torch.Tensor):
            v = value.detach()
            ident = ("tensor", str(v.device), v.data_ptr(), str(v.dtype), tuple(v.shape), tuple(v.stride()))
            if ident not in ref_of:
                if v.is_cuda:
                    bufs = on_dev.setdefault(v.device, [])
                    bufs.append(v.contiguous())
                    ref_of[ident] = (v.device, len(bufs) - 1)
                else:
                    raw = np.ascontiguousarray(v.contiguous().numpy()).reshape(-1).view(np.uint8)
                    ref_of[ident] = _finish(*_lanes_host(raw), raw.size)
            snap[key] = (str(v.dtype).replace("torch.", ""), tuple(v.shape), ident)
        elif isinstance(value, np.ndarray):
            ident = ("array", value.__array_interface__["data"][0], str(value.dtype), value.shape, value.strides)
            if ident not in ref_of:
                raw = np.ascontiguousarray(value).reshape(-1).view(np.uint8)
                ref_of[ident] = _finish(*_lanes_host(raw), raw.size)
            snap[key] = (str(value.dtype), tuple(value.shape), ident)
    lanes = {}
    for dev, bufs in on_dev.items():
        out = torch.empty((len(bufs), 2), dtype=torch.int64, device=dev)
        for i, t in enumerate(bufs):
            _device_lanes(t, out, i)
        lanes[dev] = out.cpu().numpy().view(np.uint64)
    for key, entry in snap.items():
        if entry[0] == "scalar":
            continue
        ref = ref_of[entry[2]]
        if isinstance(ref, tuple):
            dev, i = ref
            t = on_dev[dev][i]
            ref = _finish(int(lanes[dev][i, 0]), int(lanes[dev][i, 1]), t.numel() * t.element_size())
        snap[key] = (entry[0], entry[1], ref)
    return snap


def _support_of(snap: Mapping[str, tuple]) -> dict[str, tuple]:
    return {k: v for k, v in snap.items() if k not in BOUNDARY_PROGNOSTICS and k not in PRIMARY_ALIASES}


def mark_complete_step_boundary(state: dict, *, mesh: Mapping[str, Any] | None = None,
                                config: Mapping[str, Any] | None = None, dt: float | None = None) -> None:
    """Bind ``state`` (in place) to its values and, where given, to the mesh, the
    configuration and the time step it continues with (state.py:194)."""
    for name in BOUNDARY_PROGNOSTICS:
        if not isinstance(state.get(name), torch.Tensor):
            raise MpasConfigError(f"complete step boundary lacks tensor {name!r}")
    snap = _snapshot(state)
    state[MARKER] = {
        "binding": BINDING,
        "state": snap,
        "support": _support_of(snap),
        "primary_aliases": {a: snap[a] for a in PRIMARY_ALIASES if a in state},
        "mesh": mesh_digest(mesh) if mesh is not None else None,
        "config": continuation_configuration_digest(config) if config is not None else None,
        "dt": float(dt) if dt is not None else None,
    }


def has_complete_step_boundary(state: Mapping[str, Any], *, mesh: Mapping[str, Any] | None = None,
                               config: Mapping[str, Any] | None = None, dt: float | None = None) -> bool:
    """True when ``state`` carries a current binding that its values still match (and the
    given mesh / configuration / time step, state.py:239)."""
    marker = state.get(MARKER)
    if not isinstance(marker, dict) or marker.get("binding") != BINDING:
        return False
    try:
        return (marker.get("state") == _snapshot(state)
                and (mesh is None or marker.get("mesh") == mesh_digest(mesh))
                and (config is None or marker.get("config") == continuation_configuration_digest(config))
                and (dt is None or marker.get("dt") == float(dt)))
    except (MpasConfigError, ValueError):
        return False


def require_unedited_boundary_support(state: Mapping[str, Any]) -> None:
    """A marked boundary may have its prognostics edited (they are re-derived from), but
    not its diagnostics or support inputs (state.py:151)."""
    marker = state.get(MARKER)
    if not isinstance(marker, dict):
        return
    if marker.get("binding") != BINDING:
        raise MpasConfigError("complete boundary binding is unsupported; reload a current restart")
    if marker.get("support") != _snapshot(state, support_only=True):
        raise MpasConfigError("complete boundary diagnostics or support inputs were edited")
    saved = marker.get("primary_aliases", {})
    for alias, primary in PRIMARY_ALIASES.items():
        if (alias in saved) != (alias in state):
            raise MpasConfigError("complete boundary diagnostic alias inventory changed")
        if alias not in saved:
            continue
        value, prim = state[alias], state.get(primary)
        # the alias may be unchanged, or follow an edit of its primary exactly
        follows = (isinstance(value, torch.Tensor) and isinstance(prim, torch.Tensor)
                   and value.dtype == prim.dtype and value.device == prim.device
                   and value.shape == prim.shape and bool(torch.equal(value, prim)))
        if not isinstance(value, torch.Tensor) or (_snapshot({alias: value}).get(alias) != saved[alias]
                                                   and not follows):
            raise MpasConfigError("complete boundary diagnostic alias was edited")


def require_boundary_continuation_identity(state: Mapping[str, Any], *, mesh: Mapping[str, Any] | None,
                                           config: Mapping[str, Any], dt: float) -> None:
    """A marked boundary continues only on the mesh, configuration and time step it was
    bound to (state.py:221).  ``mesh`` None: a state that is its own mesh, which matches
    only a boundary bound to no mesh."""
    marker = state.get(MARKER)
    if not isinstance(marker, dict):
        return
    mesh_id = mesh_digest(mesh) if mesh is not None else None
    if (marker.get("binding") != BINDING or marker.get("mesh") != mesh_id
            or marker.get("config") != continuation_configuration_digest(config)
            or marker.get("dt") != float(dt)):
        raise MpasConfigError("complete boundary continuation identity mismatch")


__all__ = ["BOUNDARY_PROGNOSTICS", "MARKER", "BINDING", "mark_complete_step_boundary", "has_complete_step_boundary",
           "require_unedited_boundary_support", "require_boundary_continuation_identity"]
