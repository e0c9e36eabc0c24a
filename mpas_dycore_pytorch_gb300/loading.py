"""The reference's loading and I/O entry points (mpas_pytorch/__init__.py ``__all__``).

* ``load_config_from_namelist`` (reference: ic_loader.py:1441) parses a Fortran namelist
  file (``&group ... /``, ``!`` comments, quoted strings, ``.true.`` / ``T`` logicals,
  Fortran ``d`` exponents) into the configuration dictionary the step takes, rejecting
  active unsupported settings, and in strict mode keys that are not namelist options.
* ``load_initial_state`` (reference: ic_loader.py:1243) builds the runtime state and mesh
  dictionaries (derived metrics, advection stencils, reconstruction coefficients, padding
  rows) from raw initial-condition and grid fields.  The fields are given as mappings of
  arrays; reading them from netCDF files needs the ``netCDF4`` package.
* ``read_history`` / ``write_history`` / ``read_restart`` / ``write_restart`` are in
  ``netcdf_io.py`` (NetCDF-3 files with the reference's schema).
"""

from __future__ import annotations

import pathlib
import re
from typing import Any, Mapping

import numpy as np
import torch

from .errors import MpasConfigError, MpasStrictModeError, MpasUnsupportedCapabilityError

PROGNOSTIC_KEYS = ("u", "w", "theta", "rho", "scalars", "qv")


def _value(text: str) -> Any:
    t = text.strip()
    if len(t) >= 2 and t[0] == t[-1] and t[0] in "'\"":
        return t[1:-1]
    low = t.lower()
    if low in (".true.", ".t.", "true", "t"):
        return True
    if low in (".false.", ".f.", "false", "f"):
        return False
    if re.fullmatch(r"[+-]?\d+", t):
        return int(t)
    num = re.sub(r"(?<=[0-9.])[dD](?=[+-]?\d)", "e", t)
    try:
        return float(num)
    except ValueError:
        return t


def parse_namelist(path: str | pathlib.Path) -> dict[str, Any]:
    """Every ``key = value`` of every group of a Fortran namelist file."""
    out: dict[str, Any] = {}
    in_group = False
    for raw in pathlib.Path(path).read_text().splitlines():
        line = raw
        # strip comments outside quotes
        quote = None
        for i, ch in enumerate(line):
            if ch in "'\"":
                quote = None if quote == ch else (ch if quote is None else quote)
            elif ch == "!" and quote is None:
                line = line[:i]
                break
        line = line.strip()
        if not line:
            continue
        if line.startswith("&"):
            in_group = True
            continue
        if line == "/":
            in_group = False
            continue
        if not in_group:
            continue
        for part in re.split(r",(?=(?:[^'\"]|'[^']*'|\"[^\"]*\")*$)", line):
            if "=" not in part:
                continue
            key, val = part.split("=", 1)
            out[key.strip()] = _value(val)
    return out


def load_config_from_namelist(namelist_path: str | pathlib.Path, *, strict: bool = True) -> dict[str, Any]:
    """Namelist -> validated configuration (defaults filled in)."""
    from .api import active_unsupported_settings, resolved_config
    path = pathlib.Path(namelist_path)
    if not path.exists():
        raise FileNotFoundError(f"Namelist file not found: {path}")
    raw = parse_namelist(path)
    unknown = sorted(k for k in raw if not k.startswith("config_"))
    if unknown:
        msg = f"Unknown namelist keys in {path}: {unknown}"
        if strict:
            raise MpasStrictModeError(msg)
        import warnings
        warnings.warn(msg, UserWarning, stacklevel=2)
    bad = active_unsupported_settings(raw)
    if bad:
        raise MpasUnsupportedCapabilityError(f"Unsupported active MPAS namelist settings in {path}: {bad}")
    cfg = resolved_config({k: v for k, v in raw.items() if k.startswith("config_")})
    cfg["config_dt"] = float(cfg["config_dt"])
    cfg["_mpas_config_validated"] = True
    return cfg


def _read_netcdf(path: pathlib.Path) -> dict[str, Any]:
    """Fields of a grid or initial-condition file: NetCDF-3 through scipy, NetCDF-4 through
    the netCDF4 package when it is installed."""
    if not path.exists():
        raise FileNotFoundError(f"file not found: {path}")
    with open(path, "rb") as fh:
        if fh.read(3) == b"CDF":
            from .netcdf_io import read_mpas_fields
            return read_mpas_fields(path)
    try:
        import netCDF4  # noqa: F401
    except ImportError as exc:
        raise MpasUnsupportedCapabilityError(
            f"reading {path} needs the netCDF4 package, which is not installed; pass the initial-condition "
            "and grid fields to load_initial_state as mappings of arrays") from exc
    import netCDF4
    out: dict[str, Any] = {}
    with netCDF4.Dataset(str(path)) as ds:
        for name, dim in ds.dimensions.items():
            out[name] = len(dim)
        for name, var in ds.variables.items():
            a = np.asarray(var[:])
            if a.ndim >= 1 and "Time" in var.dimensions[:1]:
                a = a[0]
            out[name] = a
    return out


def load_initial_state(init_path, grid_path, mesh_support_path=None, *, device: str | torch.device = "cpu",
                       config: Mapping[str, Any] | None = None) -> tuple[dict[str, Any], dict[str, Any]]:
    """(state, mesh) runtime dictionaries from raw initial-condition and grid fields
    (mappings, or netCDF paths when netCDF4 is installed); tensors on ``device``."""
    from .api import reject_unsupported_request
    from .loader import load_arrays
    reject_unsupported_request(None, None, config)
    init = init_path if isinstance(init_path, Mapping) else _read_netcdf(pathlib.Path(init_path))
    grid = grid_path if isinstance(grid_path, Mapping) else _read_netcdf(pathlib.Path(grid_path))
    if mesh_support_path is not None:
        support = mesh_support_path if isinstance(mesh_support_path, Mapping) else \
            _read_netcdf(pathlib.Path(mesh_support_path))
        grid = dict(grid)
        for k, v in support.items():
            grid.setdefault(k, v)
    for name, src in (("nCells", grid), ("nEdges", grid), ("nVertices", grid)):
        if name not in src:
            from .errors import MpasMissingFieldError
            raise MpasMissingFieldError(fields=(name,), source="grid")
    if "theta" not in init:
        from .errors import MpasMissingFieldError
        raise MpasMissingFieldError(fields=("theta",), source="init")
    merged = load_arrays(init, grid, config, as_torch=False)
    dev = torch.device(device)

    def conv(v):
        if isinstance(v, np.ndarray):
            return torch.from_numpy(np.ascontiguousarray(v)).to(dev)
        return v

    state = {k: conv(merged[k]) for k in PROGNOSTIC_KEYS if k in merged}
    mesh = {k: conv(v) for k, v in merged.items() if k not in state}
    for k in ("num_scalars", "moist_start", "moist_end", "nCells", "nEdges", "nVertices", "nVertLevels"):
        if k in merged:
            state[k] = merged[k]
    return state, mesh


from .netcdf_io import read_history, read_restart, write_history, write_restart  # noqa: E402,F401
