"""Generate the golden fixtures under tests/golden/ by running the reference itself.

This script is the only place that executes the reference (mpas_pytorch, pure
Python + PyTorch, CPU float64).  It needs the reference source tree, named by the
environment variable ``MPAS_REFERENCE`` (the directory that holds ``mpas_pytorch/``;
there is no default), and runs in a container
without netCDF4, so it puts a two-name stub module on ``sys.path`` first (the
reference imports netCDF4 at package import, ``utils/checkpoint_reader.py:13``,
but the dynamics never touch it).

For each case it
  1. builds the raw MPAS grid/init arrays with ``mpas_dycore_pytorch_gb300.cases``;
  2. feeds them through the reference's own ``load_initial_state``
     (``ic_loader.py:1243``) by replacing ``load_checkpoint`` with an in-memory reader;
  3. runs ``run_simulation`` (``atmosphere_model.py:1474``) for ``nsteps`` steps,
     recording the prepared boundary (``on_initial``), the state after each step
     (``on_step``) and, for the first large step, the inputs and outputs of every
     stage call the step driver makes (``profiled_call`` in
     ``dynamics/time_integration.py``; the tendency stage through
     ``pack_dynamics_tendency_numeric_outputs``, ``dyn_tend.py:11239``).

Outputs: ``<case>_state.npz`` (prepared/step boundaries), ``<case>_taps.npz`` (stage
arrays) and ``<case>.json`` (config, dims, scalar stage arguments, tap index).

Run:  MPAS_REFERENCE=<reference tree> python tests/golden/make_golden.py [case ...]
"""

from __future__ import annotations

import json
import os
import pathlib
import sys
import tempfile

os.environ["PYTHONDONTWRITEBYTECODE"] = "1"
os.environ.setdefault("ATEN_CPU_CAPABILITY", "default")

HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parent.parent


def _reference_root() -> pathlib.Path:
    """The reference source tree, from ``MPAS_REFERENCE`` (required)."""
    root = os.environ.get("MPAS_REFERENCE")
    if not root:
        raise SystemExit("set MPAS_REFERENCE to the reference source tree (the directory holding mpas_pytorch/)")
    path = pathlib.Path(root)
    if not (path / "mpas_pytorch").is_dir():
        raise SystemExit(f"MPAS_REFERENCE={root!r} does not hold mpas_pytorch/")
    return path

_STUB = '''
class Dataset:
    def __init__(self, *a, **k):
        raise RuntimeError("netCDF4 stub: no file I/O")
class Variable:
    pass
__version__ = "0.0-stub"
'''


# A read-only stand-in for the netCDF4 package (absent here; the reference pins 1.7.4): the
# part of its documented API the reference's CheckpointReader uses -- Dataset(path, "r") as
# a context manager, .variables / .dimensions, a variable's [:] (native byte order), dtype,
# shape, size and dimensions -- over scipy's NetCDF-3 reader.  make_golden_files.py uses it
# so that the reference's own load_initial_state reads the case files this package writes.
_READER_STUB = '''
import numpy as _np
from scipy.io import netcdf_file as _netcdf_file

class Variable:
    def __init__(self, v):
        self._v = v
        self.dimensions = tuple(v.dimensions)
        self.shape = tuple(v.shape)
        self.dtype = v.data.dtype.newbyteorder("=")
        self.size = int(_np.prod(self.shape)) if self.shape else 1
    def __getitem__(self, idx):
        a = _np.asarray(self._v.data)
        a = a.astype(a.dtype.newbyteorder("="))
        return _np.array(a) if a.ndim == 0 else _np.array(a[idx])

class _Dim:
    def __init__(self, n):
        self.size = n
    def __len__(self):
        return self.size

class Dataset:
    def __init__(self, path, mode="r", **kw):
        if mode != "r":
            raise RuntimeError("netCDF4 stand-in: read-only")
        self._f = _netcdf_file(str(path), "r", mmap=False)
        self.variables = {k: Variable(v) for k, v in self._f.variables.items()}
        self.dimensions = {k: _Dim(n if n is not None else 1) for k, n in self._f.dimensions.items()}
    def close(self):
        self._f.close()
    def __enter__(self):
        return self
    def __exit__(self, *a):
        self.close()

__version__ = "0.0-scipy-netcdf3-reader"
'''


def _import_reference(stub: str = _STUB):
    # the reference tree is read-only input: no bytecode caches written into it (the
    # environment variable only reaches child processes)
    sys.dont_write_bytecode = True
    stub_dir = pathlib.Path(tempfile.mkdtemp(prefix="ncstub_"))
    (stub_dir / "netCDF4").mkdir()
    (stub_dir / "netCDF4" / "__init__.py").write_text(stub)
    sys.path.insert(0, str(stub_dir))
    sys.path.insert(0, str(_reference_root()))
    sys.path.insert(0, str(REPO))
    import mpas_pytorch  # noqa: F401
    return mpas_pytorch


CASES = {
    # like the level-4 CPU-runnable case: uniform levels, one cosine-bell tracer, non-monotone transport
    "g2_explicit": dict(spec=dict(level=2, nlev=12, seed=0, n_bumps=8, n_tracers=1),
                        config=dict(config_monotonic=False), dt=1800.0, nsteps=2),
    # like the level-6 headline case: stretched levels, three tracers, monotone transport
    "g2_mono": dict(spec=dict(level=2, nlev=12, dz_bottom=400.0, seed=1, n_bumps=8, n_tracers=3),
                    config=dict(config_monotonic=True), dt=1800.0, nsteps=2),
    # moist: water vapour as scalar 0 (moist coefficients cqw / cqu != 1, theta_m != theta)
    "g2_moist": dict(spec=dict(level=2, nlev=12, dz_bottom=400.0, seed=2, n_bumps=6, n_tracers=1,
                               qv_surface=0.012),
                     config=dict(config_monotonic=True), dt=1200.0, nsteps=2),
    # second-order Runge-Kutta (config_time_integration_order = 2), four acoustic substeps
    "g2_rk2": dict(spec=dict(level=2, nlev=12, seed=3, n_bumps=6, n_tracers=2),
                   config=dict(config_monotonic=False, config_time_integration_order=2,
                               config_number_of_sub_steps=4), dt=900.0, nsteps=2),
    # fixed-coefficient horizontal mixing (del2 and del4) with vertical mixing of u, w, theta
    "g2_fixed": dict(spec=dict(level=2, nlev=12, dz_bottom=400.0, seed=4, n_bumps=6, n_tracers=1,
                               w_sine=0.05),
                     config=dict(config_monotonic=True, config_horiz_mixing="2d_fixed",
                                 config_h_mom_eddy_visc4=1.0e10, config_h_theta_eddy_visc4=5.0e9,
                                 config_h_theta_eddy_visc2=2.0e4, config_v_mom_eddy_visc2=1.0,
                                 config_v_theta_eddy_visc2=1.0), dt=1200.0, nsteps=2),
    # CAM-style second-order damping in the top levels with full APVM upwinding
    "g2_cam": dict(spec=dict(level=2, nlev=12, seed=5, n_bumps=6, n_tracers=1),
                   config=dict(config_monotonic=False, config_mpas_cam_coef=1.0,
                               config_number_cam_damping_levels=4,
                               config_apvm_upwinding=1.0), dt=1200.0, nsteps=2),
    # two dynamics substeps per transport step
    "g2_split2": dict(spec=dict(level=2, nlev=12, seed=6, n_bumps=6, n_tracers=2),
                      config=dict(config_monotonic=True, config_dynamics_split_steps=2), dt=1200.0, nsteps=2),
    # coupled transport: scalars advanced inside every RK stage of the single dynamics step
    "g2_coupled": dict(spec=dict(level=2, nlev=12, seed=7, n_bumps=6, n_tracers=2),
                       config=dict(config_monotonic=True, config_split_dynamics_transport=False),
                       dt=600.0, nsteps=2),
    # Rayleigh damping of u on the top levels, vertical mixing of the perturbation from the
    # initial profiles (config_mix_full = false)
    "g2_rayleigh": dict(spec=dict(level=2, nlev=12, dz_bottom=400.0, seed=10, n_bumps=6, n_tracers=1,
                                  w_sine=0.05, uv_init=(15.0, 2.0)),
                        config=dict(config_monotonic=False, config_rayleigh_damp_u=True,
                                    config_rayleigh_damp_u_timescale_days=0.5,
                                    config_number_rayleigh_damp_u_levels=4, config_mix_full=False,
                                    config_v_mom_eddy_visc2=2.0, config_v_theta_eddy_visc2=2.0),
                        dt=1200.0, nsteps=2),
    # terrain-following levels over a 1500 m cosine hill (zz != 1, edge slopes zb / zb3 / zxu)
    "g2_terrain": dict(spec=dict(level=2, nlev=12, dz_bottom=400.0, seed=15, n_bumps=6, n_tracers=1,
                                 terrain=1500.0),
                       config=dict(config_monotonic=False), dt=1200.0, nsteps=2),
    # positive-definite limiter instead of monotonic (same limited last stage); boundaries only
    "g2_posdef": dict(spec=dict(level=2, nlev=12, seed=8, n_bumps=6, n_tracers=2),
                      config=dict(config_monotonic=False, config_positive_definite=True),
                      dt=1200.0, nsteps=2, taps=False),
    # scalar transport switched off (config_scalar_advection = false); boundaries only
    "g2_noadv": dict(spec=dict(level=2, nlev=12, seed=9, n_bumps=6, n_tracers=2),
                     config=dict(config_monotonic=True, config_scalar_advection=False),
                     dt=1200.0, nsteps=2, taps=False),
}

BASE_CONFIG = {
    "config_time_integration_order": 3,
    "config_len_disp": 120000.0,
    "config_number_of_sub_steps": 2,
    "config_dynamics_split_steps": 3,
}


def _np(v):
    import torch
    return v.detach().cpu().numpy().copy() if isinstance(v, torch.Tensor) else v


def _scalar(v):
    import numpy as np
    import torch
    if isinstance(v, torch.Tensor) and v.ndim == 0:
        return v.item()
    if isinstance(v, (bool, int, float, str)) or v is None:
        return v
    if isinstance(v, (np.integer, np.floating)):
        return v.item()
    return Ellipsis


def load_reference_case(mp, case: dict):
    """The case's raw arrays through the reference's own loader: (state, mesh, config)."""
    import numpy as np
    import torch

    import mpas_pytorch.ic_loader as icl
    from mpas_dycore_pytorch_gb300.cases import CaseSpec, make_case

    spec = CaseSpec(**case["spec"])
    init, mesh = make_case(spec)

    def to_torch(d):
        out = {}
        for k, v in d.items():
            if isinstance(v, np.ndarray):
                out[k] = torch.from_numpy(v.copy())
            elif isinstance(v, (int, np.integer)):
                out[k] = torch.tensor(int(v), dtype=torch.int32)
            else:
                out[k] = torch.tensor(float(v), dtype=torch.float64)
        return out

    tmp = pathlib.Path(tempfile.mkdtemp())
    (tmp / "init.nc").write_bytes(b"")
    (tmp / "grid.nc").write_bytes(b"")
    raw = {str(tmp / "init.nc"): to_torch(init), str(tmp / "grid.nc"): to_torch(mesh)}
    icl.load_checkpoint = lambda path, validated_fields=None, **kw: {
        k: v.clone() for k, v in raw[str(path)].items()}

    cfg = dict(BASE_CONFIG)
    cfg.update(case["config"])
    cfg["config_dt"] = case["dt"]
    state, meshd = mp.load_initial_state(tmp / "init.nc", tmp / "grid.nc", config=cfg)
    return state, meshd, cfg


def run_case(mp, name: str, case: dict) -> None:
    import numpy as np
    import torch

    import mpas_pytorch.dynamics.dyn_tend as dyn_tend_mod
    import mpas_pytorch.dynamics.time_integration as ti

    state, meshd, cfg = load_reference_case(mp, case)

    arrays: dict[str, np.ndarray] = {}
    meta: dict = {"spec": case["spec"], "config": cfg, "dt": case["dt"],
                  "nsteps": case["nsteps"], "torch": torch.__version__, "taps": []}
    for key, value in state.items():
        if isinstance(value, torch.Tensor):
            arrays[f"loaded/{key}"] = _np(value)
        elif _scalar(value) is not Ellipsis:
            meta.setdefault("loaded_scalars", {})[key] = _scalar(value)

    taps: dict[str, np.ndarray] = {}
    recording = {"on": case.get("taps", True)}
    counts: dict[str, int] = {}
    keep_per_stage = {"mpas.acoustic_step_acoustic_step": 3, "mpas.divergence_damping": 2,
                      "mpas.large_step_recovery_recover_large_step": 3,
                      "mpas.diagnostic_solve_solve_diagnostics": 3,
                      "mpas.dynamics_tendency_dyn_tend": 3,
                      "mpas.vertical_implicit_coefficients_vert_imp_coefs": 2,
                      "mpas.explicit_scalar_transport_advance_scalars_transport": 3,
                      "mpas.monotonic_scalar_transport_advance_scalars_mono_transport": 1}

    def record(stage: str, kwargs: dict, out: dict) -> None:
        i = counts.get(stage, 0)
        counts[stage] = i + 1
        if not recording["on"] or i >= keep_per_stage.get(stage, 1):
            return
        entry = {"stage": stage, "index": i, "scalars": {}, "arrays_in": [], "arrays_out": [],
                 "static_in": []}
        prefix = f"{stage}/{i}"
        for k, v in kwargs.items():
            if isinstance(v, torch.Tensor):
                a = _np(v)
                ref = arrays.get(f"loaded/{k}")
                if ref is not None and ref.shape == a.shape and ref.dtype == a.dtype \
                        and np.array_equal(ref, a):
                    entry["static_in"].append(k)  # identical to the loaded mesh/static array
                    continue
                taps[f"{prefix}/in/{k}"] = a
                entry["arrays_in"].append(k)
            else:
                s = _scalar(v)
                if s is not Ellipsis:
                    entry["scalars"][k] = s
        for k, v in out.items():
            if isinstance(v, torch.Tensor):
                taps[f"{prefix}/out/{k}"] = _np(v)
                entry["arrays_out"].append(k)
            else:
                s = _scalar(v)
                if s is not Ellipsis:
                    entry["scalars"]["out:" + k] = s
        meta["taps"].append(entry)

    orig_profiled = ti.profiled_call

    snapshots: dict[int, torch.Tensor] = {}

    def profiled(name, config, fn, *args, **kwargs):
        # stages update some inputs in place: record the values they were called with
        snapshots.clear()
        for v in list(args) + list(kwargs.values()):
            if isinstance(v, torch.Tensor):
                snapshots[id(v)] = v.detach().clone()
        before = {k: snapshots.get(id(v), v) for k, v in kwargs.items()}
        out = orig_profiled(name, config, fn, *args, **kwargs)
        if name in ("mpas.dynamics_tendency_dyn_tend", "mpas.rk_integration_setup"):
            return out
        if isinstance(out, dict):
            record(name, before, out)
        return out

    ti.profiled_call = profiled
    orig_pack = dyn_tend_mod.pack_dynamics_tendency_numeric_outputs

    def pack(compact, call_arguments, *a, **k):
        out = orig_pack(compact, call_arguments, *a, **k)
        args = {kk: snapshots.get(id(vv), vv) for kk, vv in call_arguments.items()
                if not kk.startswith("_")}
        record("mpas.dynamics_tendency_dyn_tend", args, out)
        return out

    dyn_tend_mod.pack_dynamics_tendency_numeric_outputs = pack

    def on_initial(s):
        for key, value in s.items():
            if isinstance(value, torch.Tensor):
                arrays[f"prepared/{key}"] = _np(value)
            elif _scalar(value) is not Ellipsis:
                meta.setdefault("prepared_scalars", {})[key] = _scalar(value)

    def on_step(i, s):
        recording["on"] = False
        for key in ("u", "w", "theta_m", "rho_zz", "scalars", "rho_p", "rtheta_p", "exner",
                    "pressure_p", "ru", "rw", "v", "divergence", "vorticity", "ke", "pv_edge",
                    "rho_edge", "h_edge", "uReconstructX", "uReconstructY", "uReconstructZ",
                    "uReconstructZonal", "uReconstructMeridional", "ur_cell", "vr_cell", "ruAvg",
                    "wwAvg", "theta", "rho"):
            if key in s and isinstance(s[key], torch.Tensor):
                arrays[f"step{i}/{key}"] = _np(s[key])

    try:
        mp.run_simulation(state, meshd, config=cfg, dt=case["dt"], nsteps=case["nsteps"],
                          on_step=on_step, on_initial=on_initial)
    finally:
        ti.profiled_call = orig_profiled
        dyn_tend_mod.pack_dynamics_tendency_numeric_outputs = orig_pack

    np.savez_compressed(HERE / f"{name}_state.npz", **arrays)
    np.savez_compressed(HERE / f"{name}_taps.npz", **taps)
    (HERE / f"{name}.json").write_text(json.dumps(meta, indent=1, default=str))
    size = sum((HERE / f).stat().st_size for f in (f"{name}_state.npz", f"{name}_taps.npz"))
    print(f"{name}: {len(arrays)} state arrays, {len(taps)} tap arrays, {size / 1e6:.1f} MB")


def main() -> None:
    mp = _import_reference()
    names = sys.argv[1:] or list(CASES)
    for name in names:
        run_case(mp, name, CASES[name])


if __name__ == "__main__":
    main()
