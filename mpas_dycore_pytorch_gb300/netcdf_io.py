"""History and restart files of the step boundary (reference: restart.py, output_writer.py,
io_schema.py).

The files are NetCDF with the reference's schema: the same global attributes
(``restart_schema``, ``restart_schema_version``, version and provenance strings, the
configuration / mesh / payload SHA-256 digests, ``complete_step_boundary``), dimension
names, variable names and dimensions, active rows only (padding rows are rebuilt on
reading, ``rho_zz``'s with 1.0), and the ``xtime`` / ``initial_time`` character
variables.  They are written in the NetCDF-3 64-bit-offset format through
``scipy.io.netcdf_file``, the NetCDF writer present where this package runs (the
reference writes NetCDF-4 through the netCDF4 package, which is absent here);
netCDF4-python reads NetCDF-3 files as well.  NetCDF-3 has no 64-bit integers and no
booleans: such arrays are stored as int32 / int8 with an ``mpas_dtype`` attribute that
restores the dtype on reading.  A NetCDF-4 (HDF5) file cannot be read without netCDF4
and is rejected with ``MpasUnsupportedCapabilityError``.

Digests are this package's: SHA-256 over a canonical encoding (little-endian array
bytes, sorted names), computed the same way on writing and reading, so a file is bound
to its payload, its configuration and its mesh.
"""

from __future__ import annotations

import hashlib
import json
import os
import pathlib
from datetime import datetime, timedelta, timezone
from numbers import Number
from typing import Any, Mapping

import numpy as np
import torch

from .errors import (MpasConfigError, MpasDeviceError, MpasMeshMismatchError, MpasMissingFieldError,
                     MpasUnsupportedCapabilityError)

PACKAGE_VERSION = "0.1.0"
# schema identity shared with the reference's files (io_schema.py:18-23)
HISTORY_SCHEMA = "MPAS-PyTorch diagnostic history schema v1"
RESTART_SCHEMA = "MPAS-PyTorch restart schema v1"
RESTART_SCHEMA_VERSION = 1
UPSTREAM_VERSION = "v8.3.1"
UPSTREAM_COMMIT = "b9090a1434b8ceb2a92fc985f4d97e7947cd95a6"
RVORD = 461.6 / 287.0  # R_v / R_d: theta = theta_m / (1 + RVORD qv)

# ---------------------------------------------------------------------------- field tables
# restart.py:43-153: the fields a restart must hold, the optional boundary snapshot and
# support fields, the acoustic carries (zero at a step boundary) and their dimensions
REGISTRY_FIELDS = ("u", "w", "rho_zz", "theta_m", "scalars", "pressure_p", "pressure_base", "rho_base", "theta_base",
                   "rho", "theta", "exner", "exner_base", "rtheta_base", "ru", "rw", "rho_p", "rtheta_p", "u_init",
                   "v_init", "t_init", "qv_init")
SNAPSHOT_FIELDS = ("v", "vorticity", "divergence", "ke", "pv_edge", "rho_edge", "ur_cell", "vr_cell", "uReconstructX",
                   "uReconstructY", "uReconstructZ", "uReconstructZonal", "uReconstructMeridional")
SUPPORT_FIELDS = ("fEdge", "rdzu", "deriv_two", "defc_a", "defc_b", "zgrid", "zxu", "cf1", "cf2", "cf3")
CARRY_FIELDS = ("ru_p", "rw_p", "rho_pp", "rtheta_pp", "rtheta_pp_old")
METADATA_FIELDS = ("_edge_ordering_mismatch", "_mesh_connectivity_preferred")
BOUNDARY_PROGNOSTICS = ("u", "w", "theta_m", "rho_zz", "scalars")

_T, _C, _E, _V, _L, _LP1, _S = "Time", "nCells", "nEdges", "nVertices", "nVertLevels", "nVertLevelsP1", "nScalars"
_GROUPS = (
    ((_T, _E, _L), ("u", "ru", "ru_p", "v", "rho_edge", "pv_edge")),
    ((_T, _C, _L), ("rho_zz", "theta_m", "pressure_p", "pressure_base", "rho_base", "theta_base", "rho", "theta",
                    "exner", "exner_base", "rtheta_base", "rho_p", "rtheta_p", "rho_pp", "rtheta_pp", "rtheta_pp_old",
                    "t_init", "divergence", "ke", "ur_cell", "vr_cell", "uReconstructX", "uReconstructY",
                    "uReconstructZ", "uReconstructZonal", "uReconstructMeridional")),
    ((_T, _C, _LP1), ("w", "rw", "rw_p")),
    ((_T, _V, _L), ("vorticity",)),
    ((_E,), ("fEdge",)),
    ((_E, _L), ("zxu",)),
    ((_C, "maxEdges"), ("defc_a", "defc_b")),
    ((_C, _LP1), ("zgrid",)),
    ((_E, "nDerivComp", "nDerivStencil"), ("deriv_two",)),
    ((_L,), ("u_init", "v_init", "qv_init", "rdzu")),
    ((), ("cf1", "cf2", "cf3")),
    ((_T, _C, _L, _S), ("scalars",)),
)
FIELD_DIMS: dict[str, tuple[str, ...]] = {name: dims for dims, names in _GROUPS for name in names}
_ROWS = {_C: "nCells", _E: "nEdges", _V: "nVertices"}

# io_schema.py:25-74 and output_writer.py:30-35: the advertised history fields
_CL = (_T, _C, _L)
HISTORY_FIELD_METADATA: dict[str, tuple[tuple[str, ...], str, str]] = {
    "u": ((_T, _E, _L), "m s-1", "Horizontal normal velocity at edges"),
    "w": ((_T, _C, _LP1), "m s-1", "Vertical velocity at vertical cell faces"),
    "theta": (_CL, "K", "Potential temperature"),
    "rho": (_CL, "kg m-3", "Dry air density"),
    "zz": (_CL, "1", "d(zeta)/dz, vertical metric term"),
    "qv": (_CL, "kg kg-1", "Water vapor mixing ratio"),
    "pressure": (_CL, "Pa", "Pressure"),
    "divergence": (_CL, "s-1", "Horizontal velocity divergence at cell center"),
    "vorticity": ((_T, _V, _L), "s-1", "Relative vorticity at vertices"),
    "ke": (_CL, "m2 s-2", "Kinetic energy at a cell center"),
    "uReconstructZonal": (_CL, "m s-1", "Zonal component of reconstructed horizontal velocity at cell centers"),
    "uReconstructMeridional": (_CL, "m s-1",
                               "Meridional component of reconstructed horizontal velocity at cell centers"),
}
MOISTURE_FIELDS = ("qv", "qc", "qr", "qi", "qs", "qg")
for _q in MOISTURE_FIELDS[1:]:
    HISTORY_FIELD_METADATA[_q] = (_CL, "kg kg-1", f"{_q} mixing ratio")


# ---------------------------------------------------------------------------- times, digests
_TIME_FORMATS = ("%Y-%m-%d_%H:%M:%S", "%Y-%m-%d_%H.%M.%S", "%Y-%m-%d %H:%M:%S")


def parse_mpas_time(value: str) -> datetime:
    """An MPAS time string (``YYYY-MM-DD_hh:mm:ss``; io_schema.py:83) as a UTC datetime."""
    for fmt in _TIME_FORMATS:
        try:
            return datetime.strptime(str(value), fmt).replace(tzinfo=timezone.utc)
        except ValueError:
            pass
    raise ValueError(f"invalid MPAS time {value!r}; expected YYYY-MM-DD_HH:MM:SS")


def format_mpas_time(value: datetime) -> str:
    return value.strftime("%Y-%m-%d_%H:%M:%S")


def initial_time_for_valid(xtime: str, model_time_seconds: float) -> str:
    return format_mpas_time(parse_mpas_time(xtime) - timedelta(seconds=float(model_time_seconds)))


def configuration_digest(config: Mapping[str, Any] | None) -> str:
    """SHA-256 of the configuration as sorted compact JSON (non-JSON values as str)."""
    text = json.dumps(dict(config or {}), sort_keys=True, separators=(",", ":"), default=str)
    return hashlib.sha256(text.encode()).hexdigest()


def continuation_configuration_digest(config: Mapping[str, Any] | None) -> str:
    """The configuration digest without private keys and execution policy."""
    return configuration_digest({k: v for k, v in (config or {}).items()
                                 if not str(k).startswith("_") and k != "gradient_checkpointing"})


def _host(a: Any) -> np.ndarray:
    if isinstance(a, torch.Tensor):
        return a.detach().cpu().contiguous().numpy()
    return np.ascontiguousarray(a)


def _le_bytes(a: np.ndarray) -> bytes:
    """The array's bytes in little-endian order (independent of how it was read)."""
    a = np.ascontiguousarray(a)
    if a.dtype.kind in "iufc" and a.dtype.itemsize > 1:
        a = a.astype(a.dtype.newbyteorder("<"), copy=False)
    return a.tobytes()


def _dtype_tag(a: np.ndarray) -> str:
    return a.dtype.newbyteorder("<").str if a.dtype.itemsize > 1 else a.dtype.str


def mesh_digest(mesh: Mapping[str, Any]) -> str:
    """SHA-256 over the mesh's numerical entries (name, dtype, shape, little-endian bytes;
    scalars as JSON), in sorted key order."""
    h = hashlib.sha256()
    n = 0
    for name in sorted(mesh):
        v = mesh[name]
        if isinstance(v, (torch.Tensor, np.ndarray)):
            a = _host(v)
            h.update(f"{name}\0{_dtype_tag(a)}\0{a.shape}\0".encode())
            h.update(_le_bytes(a))
            n += 1
        elif isinstance(v, (bool, int, float, str, np.generic)):
            item = v.item() if isinstance(v, np.generic) else v
            h.update(f"{name}\0scalar\0{json.dumps(item, default=str)}\0".encode())
            n += 1
    if n == 0:
        raise ValueError("mesh digest requires at least one numerical identifier")
    return h.hexdigest()


def boundary_prognostics_digest(state: Mapping[str, Any], dims: Mapping[str, int]) -> str:
    """SHA-256 of the active rows of the boundary prognostics (u, w, theta_m, rho_zz,
    scalars)."""
    h = hashlib.sha256()
    for name in BOUNDARY_PROGNOSTICS:
        a = _active(name, _host(state[name]), dims)
        h.update(f"{name}\0{_dtype_tag(a)}\0{a.shape}\0".encode())
        h.update(_le_bytes(a))
    return h.hexdigest()


def _runtime_device_dtype(state: Mapping[str, Any]) -> tuple[str, str]:
    for name in ("u", "w", "theta_m", "rho_zz", "scalars", *state):
        v = state.get(name)
        if isinstance(v, torch.Tensor) and v.is_floating_point():
            return str(v.device), str(v.dtype).replace("torch.", "")
        if isinstance(v, np.ndarray) and v.dtype.kind == "f":
            return "cpu", str(v.dtype)
    return "unknown", "unknown"


def _scientific(name: str, a: np.ndarray) -> np.ndarray:
    if a.dtype != np.float64:
        raise MpasConfigError(f"{name}: scientific data must be float64, got {a.dtype}")
    if not np.isfinite(a).all():
        raise MpasConfigError(f"{name}: scientific data must be finite")
    return a


# ---------------------------------------------------------------------------- the payload
class _Payload:
    """A NetCDF dataset in memory: global attributes, dimensions, variables."""

    def __init__(self):
        self.attrs: dict[str, Any] = {}
        self.dims: dict[str, tuple[int, bool]] = {}  # name -> (size, unlimited)
        self.vars: dict[str, tuple[tuple[str, ...], np.ndarray, dict[str, Any]]] = {}

    def digest(self, skip: str) -> str:
        """SHA-256 of everything but the attribute ``skip`` (restart.py:349 binds the same
        parts: attributes, dimensions, variables with their dimensions, dtypes, shapes,
        bytes and attributes)."""
        h = hashlib.sha256()
        for name in sorted(self.attrs):
            if name != skip:
                h.update(json.dumps([name, self.attrs[name]], allow_nan=False).encode())
        for name in sorted(self.dims):
            size, unlimited = self.dims[name]
            h.update(json.dumps([name, size, unlimited]).encode())
        for name in sorted(self.vars):
            dims, a, attrs = self.vars[name]
            if a.dtype.kind == "f" and not np.isfinite(a).all():
                raise MpasConfigError(f"field {name!r} has nonfinite data")
            h.update(json.dumps([name, list(dims), _dtype_tag(a), list(a.shape)]).encode())
            h.update(_le_bytes(a))
            for k in sorted(attrs):
                h.update(json.dumps([k, attrs[k]], default=str).encode())
        return h.hexdigest()


def _canon(v: Any) -> Any:
    if isinstance(v, bytes):
        return v.decode("utf-8")
    if isinstance(v, np.ndarray):
        if v.dtype.kind in "SU":
            return b"".join(v.ravel().tolist()).decode("utf-8") if v.dtype.kind == "S" else "".join(v.ravel())
        return v.item() if v.size == 1 else v.tolist()
    if isinstance(v, np.generic):
        return v.item()
    return v


def _storable(name: str, a: np.ndarray) -> tuple[np.ndarray, dict[str, Any]]:
    """The array in a NetCDF-3 type, with the attribute that restores its dtype."""
    kind = a.dtype.kind
    if kind == "b":
        return a.astype(np.int8), {"mpas_dtype": "bool"}
    if kind in "iu" and a.dtype not in (np.dtype(np.int8), np.dtype(np.int16), np.dtype(np.int32)):
        if a.size and (a.min() < np.iinfo(np.int32).min or a.max() > np.iinfo(np.int32).max):
            raise MpasConfigError(f"{name}: integer values exceed the 32-bit range of the file format")
        return a.astype(np.int32), {"mpas_dtype": str(a.dtype)}
    if kind == "f" and a.dtype not in (np.dtype(np.float32), np.dtype(np.float64)):
        return a.astype(np.float64), {"mpas_dtype": str(a.dtype)}
    if kind not in "iufS":
        raise MpasConfigError(f"{name}: dtype {a.dtype} cannot be stored")
    return a, {}


def _restored(a: np.ndarray, attrs: Mapping[str, Any]) -> np.ndarray:
    tag = attrs.get("mpas_dtype")
    if tag is None:
        return a
    return a.astype(bool) if tag == "bool" else a.astype(np.dtype(tag))


def _write_payload(p: _Payload, path: pathlib.Path) -> None:
    from scipy.io import netcdf_file
    f = netcdf_file(str(path), "w", version=2)
    try:
        for name, value in p.attrs.items():
            setattr(f, name, np.int32(value) if isinstance(value, (bool, int)) and not isinstance(value, str)
                    else (np.float64(value) if isinstance(value, float) else value))
        for name, (size, unlimited) in p.dims.items():
            f.createDimension(name, None if unlimited else size)
        for name, (dims, a, attrs) in p.vars.items():
            v = f.createVariable(name, "c" if a.dtype.kind == "S" else a.dtype, dims)
            if dims and p.dims[dims[0]][1]:  # a record variable grows along its first axis
                v[0:a.shape[0]] = a
            else:
                v[...] = a
            for k, val in attrs.items():
                setattr(v, k, val)
        f.flush()
    finally:
        f.close()


def _read_payload(path: pathlib.Path) -> _Payload:
    with open(path, "rb") as fh:
        magic = fh.read(4)
    if magic[:3] != b"CDF":
        raise MpasUnsupportedCapabilityError(
            f"{path} is not a NetCDF-3 file (NetCDF-4 / HDF5 files need the netCDF4 package, which is not "
            "installed here)")
    from scipy.io import netcdf_file
    p = _Payload()
    f = netcdf_file(str(path), "r", mmap=False)
    try:
        p.attrs = {k: _canon(v) for k, v in f._attributes.items()}
        nrec = None
        for name, var in f.variables.items():
            if var.isrec:
                nrec = int(var.data.shape[0])
        for name, size in f.dimensions.items():
            p.dims[name] = (int(nrec or 0) if size is None else int(size), size is None)
        for name, var in f.variables.items():
            a = np.array(var.data, copy=True)
            if a.dtype.kind in "iuf" and a.dtype.itemsize > 1:
                a = a.astype(a.dtype.newbyteorder("="))
            p.vars[name] = (tuple(var.dimensions), a, {k: _canon(v) for k, v in var._attributes.items()})
    finally:
        f.close()
    return p


class _AtomicPath:
    """Write to a temporary file beside ``path``, then rename it over ``path``."""

    def __init__(self, path: pathlib.Path, clobber: bool):
        if path.exists() and not clobber:
            raise FileExistsError(f"file already exists: {path}")
        self.path = path
        self.tmp = path.with_name(f".{path.name}.{os.getpid()}.tmp")

    def __enter__(self) -> pathlib.Path:
        return self.tmp

    def __exit__(self, exc_type, exc, tb) -> None:
        if exc_type is None:
            os.replace(self.tmp, self.path)
        elif self.tmp.exists():
            self.tmp.unlink()


def _encode_char64(text: str) -> np.ndarray:
    if len(text) > 64:
        raise MpasConfigError(f"time string exceeds 64 chars: {text!r}")
    try:
        raw = text.ljust(64).encode("ascii")
    except UnicodeEncodeError as exc:
        raise MpasConfigError(f"time string must be ASCII: {text!r}") from exc
    return np.frombuffer(raw, dtype="S1").copy()


def _decode_chars(a: np.ndarray) -> str:
    return b"".join(np.asarray(a).reshape(-1).tolist()).decode("ascii").rstrip()


# ---------------------------------------------------------------------------- active rows
def _dims_of(mesh: Mapping[str, Any], state: Mapping[str, Any]) -> dict[str, int]:
    def get(k):
        v = mesh.get(k, state.get(k, 0))
        return int(v.item() if hasattr(v, "item") else v)
    return {k: get(k) for k in ("nCells", "nEdges", "nVertices", "nVertLevels")}


def _active(name: str, a: np.ndarray, n: Mapping[str, int]) -> np.ndarray:
    """The active rows (and levels) of a known field (restart.py:235)."""
    dims = FIELD_DIMS[name]
    body = dims[1:] if dims[:1] == (_T,) else dims
    idx = []
    for d in body:
        if d in _ROWS:
            idx.append(slice(0, n[_ROWS[d]]))
        elif d == _L:
            idx.append(slice(0, n["nVertLevels"]))
        elif d == _LP1:
            idx.append(slice(0, n["nVertLevels"] + 1))
        else:
            idx.append(slice(None))
    return np.ascontiguousarray(a[tuple(idx)]) if idx else a


def _padded(name: str, a: np.ndarray, n: Mapping[str, int]) -> np.ndarray:
    """A known field with its padding row restored (zeros; restart.py:608)."""
    dims = FIELD_DIMS[name]
    body = dims[1:] if dims[:1] == (_T,) else dims
    if not body or body[0] not in _ROWS:
        return a
    out = np.zeros((a.shape[0] + 1,) + a.shape[1:], dtype=a.dtype)
    out[: a.shape[0]] = a
    return out


def _is_scalar_value(v: Any) -> bool:
    return isinstance(v, (bool, Number, np.generic)) and not isinstance(v, complex)


def _is_complete_boundary(state: Mapping[str, Any]) -> bool:
    """A step boundary as run_simulation returns it: the prepared fields plus the boundary
    snapshot and the averaged fluxes."""
    need = ("theta_m", "rho_zz", "rtheta_p", "exner", "pv_edge", "v") + SNAPSHOT_FIELDS + ("ruAvg", "wwAvg")
    return all(isinstance(state.get(k), (torch.Tensor, np.ndarray)) for k in need)


# ---------------------------------------------------------------------------- restart
def write_restart(state: Mapping[str, Any], mesh: Mapping[str, Any], path: str | os.PathLike, xtime: str, *,
                  initial_time: str | None = None, config: Mapping[str, Any] | None = None, dt: float | None = None,
                  model_time_seconds: float = 0.0, source_provenance: str = "caller-provided in-memory state",
                  clobber: bool = False) -> None:
    """Write a restart file of a step boundary (reference: restart.py:383).

    Tensors may live on the GPU (they are copied to the host).  Required fields come from
    ``state`` or ``mesh``; every other tensor or number of ``state`` is kept as an extra
    variable.  The file is written beside ``path`` and renamed over it, after it has been
    read back and checked."""
    path = pathlib.Path(path)
    if path.exists() and not clobber:
        raise FileExistsError(f"Restart file already exists: {path}")
    missing = sorted(k for k in REGISTRY_FIELDS if k not in state and k not in mesh)
    if missing:
        raise MpasMissingFieldError(fields=tuple(missing), source="restart state")
    snapshot = _is_complete_boundary(state)
    for k in CARRY_FIELDS:  # restart.py:183: a mid-RK3 savepoint is ambiguous
        v = state.get(k)
        if isinstance(v, (torch.Tensor, np.ndarray)) and not snapshot and bool(np.any(_host(v) != 0)):
            raise MpasConfigError(f"write_restart cannot serialize mid-RK3 substep state: field {k!r} is non-zero.")
    # only a boundary bound by run_simulation / run_timestep (or read from a complete
    # restart) and unedited since is written as a complete boundary (restart.py:403-416)
    from .boundary import MARKER, has_complete_step_boundary
    complete = has_complete_step_boundary(state)
    if MARKER in state and not complete:
        raise MpasConfigError("write_restart cannot save an edited timestep boundary with stale diagnostics; "
                              "advance it through run_timestep before saving the resulting complete boundary.")
    # the binding holds the full configuration (defaults filled in) the boundary was run with
    from .api import resolved_config
    if complete and not has_complete_step_boundary(state, mesh=mesh, dt=dt,
                                                   config=resolved_config(config) if config is not None else None):
        raise MpasConfigError("complete boundary continuation identity mismatch")
    if complete and not snapshot:
        missing = [k for k in SNAPSHOT_FIELDS + ("ruAvg", "wwAvg") if k not in state]
        raise MpasMissingFieldError(fields=tuple(missing), source="complete restart boundary")
    try:
        timestep = float(dt if dt is not None else (config or {}).get("config_dt", 0.0))
    except (TypeError, ValueError) as exc:
        raise MpasConfigError("restart timestep is malformed") from exc
    if not np.isfinite(timestep) or timestep < 0.0 or (complete and timestep == 0.0):
        raise MpasConfigError("restart timestep must be finite and positive for continuation")
    if dt is not None and not (np.isfinite(dt) and dt > 0.0):
        raise MpasConfigError("restart timestep must be finite and positive")
    if not np.isfinite(model_time_seconds) or model_time_seconds < 0.0:
        raise MpasConfigError("model_time_seconds must be finite and nonnegative")
    try:
        xtime = format_mpas_time(parse_mpas_time(xtime))
        initial_time = format_mpas_time(parse_mpas_time(
            initial_time if initial_time is not None else initial_time_for_valid(xtime, model_time_seconds)))
    except ValueError as exc:
        raise MpasConfigError(str(exc)) from exc

    n = _dims_of(mesh, state)
    scalars = _host(state["scalars"] if "scalars" in state else mesh["scalars"])
    p = _Payload()
    device, dtype = _runtime_device_dtype(state)
    p.attrs.update(restart_schema=RESTART_SCHEMA, restart_schema_version=RESTART_SCHEMA_VERSION,
                   package_version=PACKAGE_VERSION, upstream_version=UPSTREAM_VERSION,
                   upstream_commit=UPSTREAM_COMMIT, runtime_dtype=dtype, runtime_device=device,
                   model_time_seconds=float(model_time_seconds), timestep_seconds=timestep,
                   configuration_sha256=configuration_digest(config))
    if complete:  # the identity the boundary is bound to (restart.py:477)
        p.attrs["continuation_configuration_sha256"] = (state[MARKER].get("config")
                                                         or continuation_configuration_digest(resolved_config(config)))
    p.attrs.update(mesh_sha256=mesh_digest(mesh), source_provenance=str(source_provenance),
                   complete_step_boundary=int(complete))
    if complete:
        p.attrs["boundary_prognostics_sha256"] = boundary_prognostics_digest(state, n)
    for name, size in ((_T, 1), (_C, n["nCells"]), (_E, n["nEdges"]), (_V, n["nVertices"]),
                       (_L, n["nVertLevels"]), (_LP1, n["nVertLevels"] + 1), (_S, int(scalars.shape[-1])),
                       ("StrLen", 64)):
        p.dims[name] = (size, False)
    d2 = state.get("deriv_two", mesh.get("deriv_two"))
    if isinstance(d2, (torch.Tensor, np.ndarray)):
        d2 = _host(d2)
        p.dims["nDerivComp"], p.dims["nDerivStencil"] = (int(d2.shape[1]), False), (int(d2.shape[2]), False)
    me = mesh.get("maxEdges", state.get("maxEdges", 0))
    if int(me) > 0:
        p.dims["maxEdges"] = (int(me), False)

    known = set(REGISTRY_FIELDS + SNAPSHOT_FIELDS + SUPPORT_FIELDS + CARRY_FIELDS + METADATA_FIELDS) | {
        "xtime", "initial_time"}
    explicit = REGISTRY_FIELDS + tuple(k for k in SNAPSHOT_FIELDS + SUPPORT_FIELDS + CARRY_FIELDS + METADATA_FIELDS
                                       if k in state or k in mesh)
    extra = tuple(k for k, v in state.items() if k not in known and (not str(k).startswith("_"))
                  and (isinstance(v, (torch.Tensor, np.ndarray)) or _is_scalar_value(v)))
    for name in explicit + extra:
        value = state.get(name, mesh.get(name))
        if name in METADATA_FIELDS and _is_scalar_value(value):
            p.vars[name] = ((), np.asarray(bool(value), dtype=np.int8), {"mpas_dtype": "bool"})
            continue
        if _is_scalar_value(value):
            a = np.asarray(value.item() if isinstance(value, np.generic) else value)
            if name in FIELD_DIMS:
                a = a.astype(np.float64)
            a, attrs = _storable(name, a)
            p.vars[name] = ((), a, attrs)
            continue
        if not isinstance(value, (torch.Tensor, np.ndarray)):
            if name in REGISTRY_FIELDS:
                raise MpasMissingFieldError(fields=(name,), source="restart state")
            continue
        a = _host(value)
        if name in FIELD_DIMS:
            a = _scientific(name, _active(name, a, n))
            dims = FIELD_DIMS[name]
            want = tuple(p.dims[d][0] for d in (dims[1:] if dims[:1] == (_T,) else dims) if d in p.dims)
            if a.shape != want or any(d not in p.dims for d in dims):
                raise MpasConfigError(f"restart field {name!r} has malformed shape {a.shape}; expected {want}")
            if dims[:1] == (_T,):
                a = a[None]
            p.vars[name] = (dims, a, {})
        else:
            if a.dtype.kind == "f" and not np.isfinite(a).all():
                raise MpasConfigError(f"restart field {name!r} has nonfinite data")
            a, attrs = _storable(name, a)
            dims = []
            for axis, size in enumerate(a.shape):
                dn = f"{name}__dim{axis}"
                p.dims.setdefault(dn, (int(size), False))
                dims.append(dn)
            p.vars[name] = (tuple(dims), a, attrs)
    p.vars["xtime"] = ((_T, "StrLen"), _encode_char64(xtime)[None], {})
    p.vars["initial_time"] = (("StrLen",), _encode_char64(initial_time), {})
    p.attrs["restart_payload_sha256"] = p.digest(skip="restart_payload_sha256")
    with _AtomicPath(path, clobber) as tmp:
        _write_payload(p, tmp)
        read_restart(tmp, mesh=mesh, config=config, dt=dt)


def _is_hex64(v: Any) -> bool:
    return isinstance(v, str) and len(v) == 64 and all(ch in "0123456789abcdef" for ch in v)


def read_restart(path: str | os.PathLike, *, mesh: Mapping[str, Any] | None = None,
                 config: Mapping[str, Any] | None = None, dt: float | None = None,
                 device: str | torch.device = "cpu") -> tuple[dict[str, Any], str]:
    """Read a restart file into a state dictionary with padding rows (reference:
    restart.py:690); returns ``(state, xtime)``.  ``device`` may be the CPU or a CUDA
    device."""
    path = pathlib.Path(path)
    if not path.exists():
        raise FileNotFoundError(f"Restart file not found: {path}")
    try:
        target = torch.device(device)
    except (TypeError, RuntimeError, ValueError) as exc:
        raise MpasDeviceError("restart loading needs a CPU or CUDA device", requested=str(device)) from exc
    if target.type not in ("cpu", "cuda"):
        raise MpasDeviceError("restart loading needs a CPU or CUDA device", requested=str(device))
    p = _read_payload(path)
    a = p.attrs
    if a.get("restart_schema_version") is None:
        raise MpasConfigError("restart schema version is missing")
    if not isinstance(a["restart_schema_version"], int) or a["restart_schema_version"] != RESTART_SCHEMA_VERSION:
        raise MpasConfigError(f"unsupported restart schema version {a['restart_schema_version']!r}; "
                              f"expected {RESTART_SCHEMA_VERSION}")
    if a.get("restart_schema") != RESTART_SCHEMA:
        raise MpasConfigError("restart schema name is missing or malformed")
    for k in ("package_version", "upstream_version", "upstream_commit", "runtime_dtype", "runtime_device",
              "model_time_seconds", "timestep_seconds", "configuration_sha256", "mesh_sha256", "source_provenance"):
        if k not in a:
            raise MpasConfigError(f"restart attribute {k!r} is missing")
    complete = a.get("complete_step_boundary")
    if not isinstance(complete, int) or complete not in (0, 1):
        raise MpasConfigError("restart complete-step boundary flag is malformed")
    digests = ["configuration_sha256", "mesh_sha256"]
    if complete:
        digests += ["continuation_configuration_sha256", "boundary_prognostics_sha256"]
    for k in digests:
        if not _is_hex64(a.get(k)):
            raise MpasConfigError(f"restart digest {k!r} is missing or malformed")
    if a["runtime_dtype"] != "float64":
        raise MpasConfigError("unsupported or missing runtime_dtype: expected 'float64'")
    try:
        timestep = float(a["timestep_seconds"])
    except (TypeError, ValueError) as exc:
        raise MpasConfigError("timestep metadata is malformed") from exc
    if not np.isfinite(timestep) or timestep < 0.0 or (complete and timestep == 0.0):
        raise MpasConfigError("timestep metadata must be finite and positive for continuation")
    if config is not None and a["configuration_sha256"] != configuration_digest(config):
        raise MpasConfigError("restart configuration digest mismatch")
    if dt is not None and timestep != float(dt):
        raise MpasConfigError("restart timestep mismatch")
    missing = sorted(k for k in REGISTRY_FIELDS if k not in p.vars)
    if missing:
        raise MpasMissingFieldError(fields=tuple(missing), source=str(path))
    if complete:
        missing = [k for k in SNAPSHOT_FIELDS + ("ruAvg", "wwAvg") if k not in p.vars]
        if missing:
            raise MpasMissingFieldError(fields=missing, source="complete restart boundary")
    for k in ("xtime", "initial_time"):
        if k not in p.vars:
            raise MpasMissingFieldError(fields=(k,), source=str(path))
    try:
        xtime = _decode_chars(p.vars["xtime"][1])
        initial_time = _decode_chars(p.vars["initial_time"][1])
        span = (parse_mpas_time(xtime) - parse_mpas_time(initial_time)).total_seconds()
        if span != float(a["model_time_seconds"]) or float(a["model_time_seconds"]) < 0.0:
            raise MpasConfigError("restart time metadata is malformed: xtime, initial_time and "
                                  "model_time_seconds are inconsistent")
    except (TypeError, ValueError, UnicodeDecodeError) as exc:
        raise MpasConfigError(f"restart time metadata is malformed: {exc}") from exc
    if a.get("restart_payload_sha256") != p.digest(skip="restart_payload_sha256"):
        raise MpasConfigError("restart boundary payload integrity digest mismatch")
    for k in (_T, _C, _E, _V, _L, _LP1, _S, "StrLen"):
        if k not in p.dims or p.dims[k][0] <= 0:
            raise MpasConfigError(f"restart dimension {k!r} is missing or empty")
    if p.dims["StrLen"][0] != 64 or p.dims[_T][0] != 1 or p.dims[_LP1][0] != p.dims[_L][0] + 1:
        raise MpasConfigError("restart time, string or vertical face dimension is malformed")
    if p.vars["xtime"][0] != (_T, "StrLen") or p.vars["initial_time"][0] != ("StrLen",):
        raise MpasConfigError("restart time string dimensions are malformed")
    n = {"nCells": p.dims[_C][0], "nEdges": p.dims[_E][0], "nVertices": p.dims[_V][0],
         "nVertLevels": p.dims[_L][0]}
    state: dict[str, Any] = dict(n)
    state["num_scalars"] = p.dims[_S][0]
    state["_restart_model_time_seconds"] = float(a["model_time_seconds"])
    if mesh is not None:
        md = _dims_of(mesh, {})
        for k in ("nCells", "nEdges", "nVertLevels"):
            if k in mesh and md[k] != n[k]:
                raise MpasMeshMismatchError(dim_name=k, init_value=n[k], grid_value=md[k])
        if a["mesh_sha256"] != mesh_digest(mesh):
            raise MpasMeshMismatchError("restart mesh digest mismatch")
        for k, v in mesh.items():
            state.setdefault(k, v)
    for name, (dims, arr, attrs) in p.vars.items():
        if name in ("xtime", "initial_time") or arr.dtype.kind in "SU":
            continue
        if name in FIELD_DIMS and dims != FIELD_DIMS[name]:
            raise MpasConfigError(f"restart field {name!r} dimensions are malformed")
        if name in FIELD_DIMS:
            _scientific(name, arr)
        arr = _restored(arr, attrs)
        if arr.ndim == 0:
            if name in METADATA_FIELDS or attrs.get("mpas_dtype") == "bool":
                state[name] = bool(arr.item())
            else:
                state[name] = arr.item()
            continue
        if name in FIELD_DIMS:
            if dims[:1] == (_T,):
                arr = arr[0]
            arr = _padded(name, arr, n)
        t = torch.from_numpy(np.ascontiguousarray(arr)).to(target)
        state[name] = t
    if isinstance(state.get("rho_zz"), torch.Tensor) and state["rho_zz"].shape[0] > n["nCells"]:
        state["rho_zz"][n["nCells"]] = 1.0  # the padding row's sentinel
    state["initial_time"] = initial_time
    if complete:
        if a["boundary_prognostics_sha256"] != boundary_prognostics_digest(state, n):
            raise MpasConfigError("restart boundary prognostic digest mismatch")
        # bound to the file's own identity digests (restart.py:961-969)
        from .boundary import MARKER, mark_complete_step_boundary
        mark_complete_step_boundary(state)
        state[MARKER].update(mesh=a["mesh_sha256"], config=a["continuation_configuration_sha256"], dt=timestep)
    return state, xtime


# ---------------------------------------------------------------------------- history
def history_scalar_fields(state: Mapping[str, Any]) -> tuple[str, ...]:
    """Names of the scalar slots (qv, qc, qr, qi, qs, qg order; output_writer.py:38)."""
    s = state.get("scalars")
    if isinstance(s, (torch.Tensor, np.ndarray)):
        if s.shape[-1] > len(MOISTURE_FIELDS):
            raise MpasConfigError("Named history scalar expansion supports qv/qc/qr/qi/qs/qg only")
        return MOISTURE_FIELDS[: s.shape[-1]]
    return tuple(k for k in MOISTURE_FIELDS if k in state)


def _history_fields(state: Mapping[str, Any], mesh: Mapping[str, Any],
                    requested: list[str] | None) -> dict[str, np.ndarray]:
    """The advertised diagnostics, active rows (output_writer.py:209): u, w, theta =
    theta_m / (1 + RVORD qv), rho = rho_zz zz, zz, qv, pressure = p' + p_base, divergence,
    ke, vorticity, the reconstructed zonal / meridional winds and the named scalars."""
    comb = dict(mesh)
    comb.update(state)
    n = _dims_of(comb, {})
    C, E, V, L = n["nCells"], n["nEdges"], n["nVertices"], n["nVertLevels"]
    if requested is not None:
        names: list[str] = []
        for k in requested:
            names.extend(history_scalar_fields(comb) if k == "scalars" else (k,))
        requested = list(dict.fromkeys(names))
        unknown = [k for k in requested if k not in HISTORY_FIELD_METADATA]
        if unknown:
            raise MpasConfigError(f"Unsupported history fields: {unknown}")
    want = (lambda k: True) if requested is None else (lambda k: k in requested)
    needs = {"u": ("u",), "w": ("w",), "theta": ("theta_m",), "rho": ("rho_zz", "zz"), "zz": ("zz",)}
    miss = sorted({x for k, xs in needs.items() if want(k) for x in xs if x not in comb})
    if miss:
        raise MpasMissingFieldError(fields=miss, source="history state")

    def h(k):
        return _host(comb[k]).astype(np.float64, copy=False)

    def qv():
        if "scalars" in comb:
            return h("scalars")[:C, :L, 0]
        if "qv" in comb:
            return h("qv")[:C, :L]
        raise MpasMissingFieldError(fields=("scalars|qv",), source="history state")

    out: dict[str, np.ndarray] = {}
    if want("u"):
        out["u"] = h("u")[:E, :L]
    if want("w"):
        out["w"] = h("w")[:C, : L + 1]
    if want("theta"):
        out["theta"] = h("theta_m")[:C, :L] / (1.0 + RVORD * qv())
    if want("rho"):
        out["rho"] = h("rho_zz")[:C, :L] * h("zz")[:C, :L]
    if want("zz"):
        out["zz"] = h("zz")[:C, :L]
    if want("qv"):
        out["qv"] = qv()
    if want("pressure") and "pressure_p" in comb and "pressure_base" in comb:
        out["pressure"] = h("pressure_p")[:C, :L] + h("pressure_base")[:C, :L]
    for k, rows in (("divergence", C), ("ke", C), ("vorticity", V)):
        if want(k) and k in comb:
            out[k] = h(k)[:rows, :L]
    for k, alias in (("uReconstructZonal", "ur_cell"), ("uReconstructMeridional", "vr_cell")):
        if want(k):
            src = k if k in comb else (alias if alias in comb else None)
            if src is not None:
                out[k] = h(src)[:C, :L]
    if requested is not None:
        names = history_scalar_fields(comb)
        for i, k in enumerate(MOISTURE_FIELDS[1:], start=1):
            if k in requested and k in names:
                out[k] = (h("scalars")[..., i] if "scalars" in comb else h(k))[:C, :L]
        missing = [k for k in requested if k not in out]
        if missing:
            raise MpasMissingFieldError(fields=missing, source="history state")
    for k, v in out.items():
        _scientific(f"history field {k!r}", np.ascontiguousarray(v))
    return {k: np.ascontiguousarray(v) for k, v in out.items()}


_RESERVED = ("history_schema", "package_version", "upstream_version", "upstream_commit", "configuration_sha256",
             "source_provenance", "runtime_dtype", "runtime_device", "timestep_seconds")


def write_history(filepath: str | os.PathLike, state: Mapping[str, Any], mesh: Mapping[str, Any], *,
                  xtime: str = "", global_attrs: Mapping[str, Any] | None = None, fields: list[str] | None = None,
                  config: Mapping[str, Any] | None = None, dt: float | None = None, model_time_seconds: float = 0.0,
                  initial_time: str | None = None, source_provenance: str = "caller-provided in-memory state",
                  clobber: bool = False) -> None:
    """Write one history file of the selected diagnostics (reference:
    output_writer.py:329)."""
    path = pathlib.Path(filepath)
    comb = dict(mesh)
    comb.update(state)
    n = _dims_of(comb, {})
    values = _history_fields(state, mesh, fields)
    try:
        valid = format_mpas_time(parse_mpas_time(xtime or "1970-01-01_00:00:00"))
        if not np.isfinite(model_time_seconds) or model_time_seconds < 0.0:
            raise MpasConfigError("model_time_seconds must be finite and nonnegative")
        ref_time = format_mpas_time(parse_mpas_time(initial_time or initial_time_for_valid(valid, model_time_seconds)))
    except (ValueError, OverflowError) as exc:
        raise MpasConfigError(str(exc)) from exc
    timestep = float(dt if dt is not None else (config or {}).get("config_dt", 0.0))
    if not np.isfinite(timestep) or timestep < 0.0:
        raise MpasConfigError("history timestep must be finite and nonnegative")
    clash = sorted(set(global_attrs or {}) & set(_RESERVED))
    if clash:
        raise MpasConfigError(f"Reserved global attributes: {clash}")
    if not values:
        raise MpasConfigError("History must contain at least one diagnostic field")
    sizes = {_T: 1, _C: n["nCells"], _E: n["nEdges"], _V: n["nVertices"], _L: n["nVertLevels"],
             _LP1: n["nVertLevels"] + 1}
    p = _Payload()
    p.dims[_T] = (1, True)
    for k in (_C, _E, _V, _L, _LP1):
        p.dims[k] = (sizes[k], False)
    p.dims["StrLen"] = (64, False)
    for k, v in values.items():
        dims, units, long_name = HISTORY_FIELD_METADATA[k]
        if v.shape != tuple(sizes[d] for d in dims[1:]):
            raise MpasConfigError(f"history field {k!r} shape {v.shape} differs from "
                                  f"{tuple(sizes[d] for d in dims[1:])}")
        p.vars[k] = (dims, v[None], {"units": units, "long_name": long_name})
    p.vars["time"] = ((_T,), np.asarray([float(model_time_seconds)]),
                      {"units": f"seconds since {ref_time.replace('_', ' ')}", "calendar": "gregorian",
                       "standard_name": "time", "long_name": "model time"})
    p.vars["xtime"] = ((_T, "StrLen"), _encode_char64(valid)[None], {"long_name": "model valid time"})
    device, dtype = _runtime_device_dtype(state)
    p.attrs.update(model_name="mpas", core_name="atmosphere", source="MPAS-Atmosphere PyTorch",
                   Conventions="CF-1.10, MPAS", history_schema=HISTORY_SCHEMA, package_version=PACKAGE_VERSION,
                   upstream_version=UPSTREAM_VERSION, upstream_commit=UPSTREAM_COMMIT, runtime_dtype=dtype,
                   runtime_device=device, timestep_seconds=timestep, configuration_sha256=configuration_digest(config),
                   source_provenance=str(source_provenance))
    for k, v in (global_attrs or {}).items():
        p.attrs[k] = v
    with _AtomicPath(path, clobber) as tmp:
        _write_payload(p, tmp)
        validate_history(tmp)


def validate_history(filepath: str | os.PathLike) -> None:
    """Check a history file against the public diagnostic schema (reference:
    output_writer.py:54)."""
    p = _read_payload(pathlib.Path(filepath))
    a = p.attrs
    for k, want in (("history_schema", HISTORY_SCHEMA), ("upstream_version", UPSTREAM_VERSION),
                    ("upstream_commit", UPSTREAM_COMMIT)):
        if a.get(k) != want:
            raise MpasConfigError(f"history {k} mismatch or missing")
    for k in ("package_version", "configuration_sha256", "source_provenance", "runtime_dtype", "runtime_device",
              "timestep_seconds"):
        if k not in a:
            raise MpasConfigError(f"history attribute {k!r} is missing")
    if a["runtime_dtype"] != "float64":
        raise MpasConfigError("unsupported or missing runtime_dtype: expected 'float64'")
    try:
        ts = float(a["timestep_seconds"])
    except (TypeError, ValueError) as exc:
        raise MpasConfigError("timestep metadata is malformed") from exc
    if not np.isfinite(ts) or ts < 0.0:
        raise MpasConfigError("timestep metadata must be finite and nonnegative")
    for k in (_C, _E, _V, _L):
        if k not in p.dims or p.dims[k][0] <= 0:
            raise MpasConfigError(f"history dimension {k!r} is missing or empty")
    if p.dims.get(_LP1, (0,))[0] != p.dims[_L][0] + 1:
        raise MpasConfigError("history vertical face dimension is malformed")
    if "time" not in p.vars or "xtime" not in p.vars:
        raise MpasConfigError("history time/xtime coordinate is missing")
    tdims, tval, tattrs = p.vars["time"]
    if tdims != (_T,) or not tattrs.get("units") or tattrs.get("standard_name") != "time":
        raise MpasConfigError("history time coordinate is malformed")
    if tattrs.get("calendar") != "gregorian":
        raise MpasConfigError("history time calendar is malformed")
    if p.vars["xtime"][0] != (_T, "StrLen"):
        raise MpasConfigError("history xtime dimensions are malformed")
    try:
        if tval.size != 1 or not np.isfinite(tval).all() or float(tval[0]) < 0.0:
            raise ValueError("time value must be one finite nonnegative number")
        units = str(tattrs["units"])
        if not units.startswith("seconds since "):
            raise ValueError(f"unsupported time units {units!r}")
        ref = parse_mpas_time(units[len("seconds since "):].strip())
        decoded = ref + timedelta(seconds=float(tval[0]))
        xt = _decode_chars(p.vars["xtime"][1][0])
        if format_mpas_time(decoded) != format_mpas_time(parse_mpas_time(xt)):
            raise ValueError("numeric time and xtime disagree")
    except (IndexError, TypeError, ValueError, OverflowError) as exc:
        raise MpasConfigError(f"history time coordinate is malformed: {exc}") from exc
    data = set(p.vars) - {"time", "xtime"}
    if not data:
        raise MpasConfigError("history contains no advertised diagnostic fields")
    for k in data:
        dims, arr, attrs = p.vars[k]
        meta = HISTORY_FIELD_METADATA.get(k)
        if meta is None:
            raise MpasConfigError(f"history field {k!r} is not advertised")
        _scientific(k, arr)
        if dims != meta[0]:
            raise MpasConfigError(f"history field {k!r} dimensions are malformed")
        if attrs.get("units") != meta[1]:
            raise MpasConfigError(f"history field {k!r} units are missing or wrong")
        if attrs.get("long_name") != meta[2]:
            raise MpasConfigError(f"history field {k!r} long_name is missing or wrong")


def read_history(filepath: str | os.PathLike, *, validate: bool = True) -> dict[str, Any]:
    """``{"fields": arrays, "dimensions": sizes (None when unlimited), "attributes":
    global attributes}`` of one history file (reference: output_writer.py:158)."""
    path = pathlib.Path(filepath)
    if validate:
        validate_history(path)
    p = _read_payload(path)
    return {"fields": {k: v[1] for k, v in p.vars.items()},
            "dimensions": {k: (None if unl else size) for k, (size, unl) in p.dims.items()},
            "attributes": dict(p.attrs)}


# ---------------------------------------------------------------------------- MPAS grid / init files
# MPAS dimension names of the grid and initial-condition fields (C order: the first axis
# is the mesh entity); time-dependent initial fields carry a leading Time axis.
_TWO, _FIFTEEN, _ME, _ME2, _VD = "TWO", "FIFTEEN", "maxEdges", "maxEdges2", "vertexDegree"
_MPAS_GROUPS = (
    ((_C,), ("nEdgesOnCell", "areaCell", "latCell", "lonCell", "xCell", "yCell", "zCell", "meshDensity",
             "indexToCellID")),
    ((_E,), ("nEdgesOnEdge", "dcEdge", "dvEdge", "latEdge", "lonEdge", "xEdge", "yEdge", "zEdge", "angleEdge", "fEdge",
             "indexToEdgeID")),
    ((_V,), ("areaTriangle", "latVertex", "lonVertex", "xVertex", "yVertex", "zVertex", "fVertex", "indexToVertexID")),
    ((_C, _ME), ("cellsOnCell", "edgesOnCell", "verticesOnCell", "defc_a", "defc_b")),
    ((_E, _TWO), ("cellsOnEdge", "verticesOnEdge")),
    ((_V, _VD), ("edgesOnVertex", "cellsOnVertex", "kiteAreasOnVertex")),
    ((_E, _ME2), ("edgesOnEdge", "weightsOnEdge")),
    ((_T, _E, _L), ("u",)),
    ((_T, _C, _LP1), ("w",)),
    ((_T, _C, _L), ("theta", "rho", "rho_base", "theta_base", "qv")),
    ((_T, _C, _L, "num_scalars"), ("scalars",)),
    ((_C, _L), ("zz", "t_init")),
    ((_C, _LP1), ("zgrid",)),
    ((_E, _TWO, _LP1), ("zb", "zb3")),
    ((_E, _L), ("zxu",)),
    ((_E, _TWO, _FIFTEEN), ("deriv_two",)),
    ((_L,), ("u_init", "v_init", "qv_init", "rdzw", "dzw", "rdzu", "dzu", "fzm", "fzp", "fnm", "fnp", "rdnw")),
)
MPAS_FIELD_DIMS: dict[str, tuple[str, ...]] = {n: d for d, names in _MPAS_GROUPS for n in names}


def write_mpas_fields(path: str | os.PathLike, fields: Mapping[str, Any], *, attrs: Mapping[str, Any] | None = None,
                      clobber: bool = False) -> None:
    """Write raw MPAS grid or initial-condition fields (mappings of arrays and numbers, as
    ``load_initial_state`` takes them) as a NetCDF-3 file with MPAS dimension names.
    Integer entries named like dimensions (``nCells``, ``maxEdges`` ...) become
    dimensions; other numbers become 0-d variables; 64-bit integers are stored as int32."""
    p = _Payload()
    sizes = {k: int(v) for k, v in fields.items() if isinstance(v, (int, np.integer)) and
             k in (_C, _E, _V, _ME, _ME2, _VD, _L)}
    arrays = {k: _host(v) for k, v in fields.items() if isinstance(v, (np.ndarray, torch.Tensor))}
    for k, a in arrays.items():  # dimensions the table implies
        for d, n in zip(MPAS_FIELD_DIMS.get(k, ())[1:] if MPAS_FIELD_DIMS.get(k, ("",))[0] == _T
                        else MPAS_FIELD_DIMS.get(k, ()), a.shape):
            sizes.setdefault(d, int(n))
    if _L in sizes:
        sizes.setdefault(_LP1, sizes[_L] + 1)
    p.dims[_T] = (1, True)
    for d, n in sizes.items():
        p.dims[d] = (n, False)
    for k, v in fields.items():
        if k in sizes:
            continue
        if isinstance(v, (np.ndarray, torch.Tensor)):
            a, vattrs = _storable(k, arrays[k])
            dims = MPAS_FIELD_DIMS.get(k)
            body = dims[1:] if dims and dims[0] == _T else dims
            if dims is None or len(body) != a.ndim or any(p.dims[d][0] != n for d, n in zip(body, a.shape)):
                dims = []
                for axis, n in enumerate(a.shape):
                    dn = next((d for d in (_C, _E, _V) if axis == 0 and p.dims.get(d, (0,))[0] == n),
                              f"{k}__dim{axis}")
                    p.dims.setdefault(dn, (int(n), False))
                    dims.append(dn)
                dims = tuple(dims)
            elif dims[0] == _T:
                a = a[None]
            p.vars[k] = (tuple(dims), a, vattrs)
        elif _is_scalar_value(v):
            a, vattrs = _storable(k, np.asarray(v.item() if isinstance(v, np.generic) else v))
            p.vars[k] = ((), a, vattrs)
    p.attrs.update(dict(attrs or {}))
    with _AtomicPath(pathlib.Path(path), clobber) as tmp:
        _write_payload(p, tmp)


def read_mpas_fields(path: str | os.PathLike) -> dict[str, Any]:
    """A NetCDF-3 grid or initial-condition file as a mapping: dimensions as ints, the
    first record of time-dependent fields, 0-d variables as numbers, and the global
    attributes that do not clash with a field."""
    p = _read_payload(pathlib.Path(path))
    out: dict[str, Any] = {}
    for k, (size, unlimited) in p.dims.items():
        if not unlimited and "__dim" not in k:
            out[k] = size
    for k, (dims, a, attrs) in p.vars.items():
        a = _restored(a, attrs)
        if a.ndim == 0:
            out[k] = a.item()
        else:
            out[k] = a[0] if dims[:1] == (_T,) else a
    for k, v in p.attrs.items():
        out.setdefault(k, v)
    return out
