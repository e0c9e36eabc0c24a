"""The reference's per-stage keyword operators on the GPU (the ``atm_*_work`` routines of
its routine map, docs/ROUTINE_MAP.md:8-25).

Each operator takes the reference routine's keyword arguments (arrays with the padding
rows, the loop bounds, the stage scalars such as ``rk_step`` or ``dts``) and returns its
outputs under the reference's names and shapes (padded, or compact where the reference
returns the active rows only), as CUDA tensors.  The stage runs through the library's
C entry point for that stage (``stages.py``).

The mesh stays resident on the device between calls: ``use_mesh(mesh, config, dt)`` loads
it once (with the configuration the stages run with), and every operator call checks that
its dimensions, its connectivity arrays and its configuration keywords are that mesh's and
that configuration's, and raises ``MpasConfigError`` otherwise.
"""

from __future__ import annotations

from typing import Any, Mapping

import numpy as np
import torch

from .errors import MpasConfigError
from .stages import PRE, STAGES, run_stage

# reference routine -> stage key of stages.STAGES, and the reference file:line
ROUTINES = {
    "atm_compute_moist_coefficients": ("moist", "dynamics/moist_coefficients.py:124"),
    "atm_compute_vert_imp_coefs_work": ("vimp", "dynamics/vert_imp_coefs.py:188"),
    "atm_compute_dyn_tend_work": ("dyn_tend", "dynamics/dyn_tend.py:10836"),
    "atm_set_smlstep_pert_variables_work": ("smlstep", "dynamics/smlstep_pert.py:373"),
    "atm_advance_acoustic_step_work": ("acoustic", "dynamics/acoustic_step.py:1297"),
    "atm_divergence_damping_3d": ("divdamp", "dynamics/divergence_damping.py:299"),
    "atm_recover_large_step_variables_work": ("recover", "dynamics/recover_large_step.py:1090"),
    "atm_compute_solve_diagnostics_work": ("diag", "dynamics/solve_diagnostics.py:1052"),
    "atm_advance_scalars_work": ("scalars", "dynamics/advance_scalars.py:1272"),
    "atm_advance_scalars_mono_work": ("scalars_mono", "dynamics/advance_scalars_mono.py:2878"),
    "mpas_reconstruct_2d": ("reconstruct", "dynamics/vector_reconstruction.py:311"),
}

# outputs the reference returns without the padding row: (stage, output) -> row dimension
_COMPACT = {("diag", "h_edge"): "nEdges", ("diag", "v"): "nEdges", ("diag", "pv_edge"): "nEdges",
            ("diag", "divergence"): "nCells", ("diag", "ke"): "nCells", ("diag", "vorticity"): "nVertices"}
_COMPACT.update({("vimp", PRE + n + "_active"): "nCells"
                 for n in ("cofwr", "cofwz", "coftz", "cofwt", "a_tri", "alpha_tri", "gamma_tri")})
# stage keywords that restate a configuration option
_OPTION_ALIASES = {"coef_3rd_order": "config_coef_3rd_order", "epssm": "config_epssm"}
_CONNECTIVITY = ("cellsOnEdge", "edgesOnCell", "nEdgesOnCell", "verticesOnEdge", "edgesOnVertex")

_context: dict[str, Any] = {}


def use_mesh(mesh: Mapping[str, Any], config: Mapping[str, Any] | None = None, dt: float | None = None,
             num_scalars: int | None = None, device: str | torch.device = "cuda"):
    """Load ``mesh`` onto the device for the keyword operators, with the configuration and
    time step their stages run with; returns the resident ``Model``."""
    from .api import Model, resolved_config
    cfg = resolved_config(config)
    dt = float(cfg["config_dt"] if dt is None else dt)
    model = Model(mesh, cfg, dt, num_scalars=num_scalars, device=device)
    _context.clear()
    _context.update(model=model, mesh=mesh)
    return model


def _host(v: Any) -> np.ndarray:
    return v.detach().cpu().numpy() if isinstance(v, torch.Tensor) else np.asarray(v)


def _same(a: Any, b: Any) -> bool:
    if isinstance(a, (bool, np.bool_)) or isinstance(b, (bool, np.bool_)):
        return bool(a) == bool(b)
    if isinstance(a, (int, float, np.number)) and isinstance(b, (int, float, np.number)):
        return float(a) == float(b)
    return a == b


def _checked_model(routine: str, kw: Mapping[str, Any]):
    model = _context.get("model")
    if model is None:
        raise MpasConfigError(f"{routine}: no resident mesh; call use_mesh(mesh, config, dt) first")
    dm = model.dmesh
    for name, n in (("nCells", dm.nCells), ("nEdges", dm.nEdges), ("nVertices", dm.nVertices),
                    ("nVertLevels", dm.nVertLevels)):
        if name in kw and int(kw[name]) != int(n):
            raise MpasConfigError(f"{routine}: {name}={int(kw[name])} but the resident mesh has {int(n)}")
    mesh = _context["mesh"]
    for name in _CONNECTIVITY:
        if name in kw and name in mesh and kw[name] is not mesh[name]:
            if not np.array_equal(_host(kw[name]), _host(mesh[name])):
                raise MpasConfigError(f"{routine}: {name} differs from the resident mesh's")
    for k, v in kw.items():
        opt = _OPTION_ALIASES.get(k, k)
        if opt.startswith("config_") and opt in model.cfg and v is not None and not isinstance(v, torch.Tensor):
            if not _same(v, model.cfg[opt]):
                raise MpasConfigError(f"{routine}: {k}={v!r} but the resident configuration has "
                                      f"{opt}={model.cfg[opt]!r}")
    return model


def _operator(routine: str):
    key, ref = ROUTINES[routine]

    def op(**kwargs):
        model = _checked_model(routine, kwargs)
        out = run_stage(model, key, kwargs)
        dm = model.dmesh
        for name, dim in _COMPACT.items():
            if name[0] == key and name[1] in out:
                out[name[1]] = out[name[1]][:int(getattr(dm, dim))]
        return out

    op.__name__ = routine
    op.__qualname__ = routine
    op.__doc__ = (f"The reference's {routine} ({ref}) on the resident mesh: its keyword arguments in, "
                  f"its outputs (CUDA tensors) out.")
    return op


atm_compute_moist_coefficients = _operator("atm_compute_moist_coefficients")
atm_compute_vert_imp_coefs_work = _operator("atm_compute_vert_imp_coefs_work")
atm_compute_dyn_tend_work = _operator("atm_compute_dyn_tend_work")
atm_set_smlstep_pert_variables_work = _operator("atm_set_smlstep_pert_variables_work")
atm_advance_acoustic_step_work = _operator("atm_advance_acoustic_step_work")
atm_divergence_damping_3d = _operator("atm_divergence_damping_3d")
atm_recover_large_step_variables_work = _operator("atm_recover_large_step_variables_work")
atm_compute_solve_diagnostics_work = _operator("atm_compute_solve_diagnostics_work")
atm_advance_scalars_work = _operator("atm_advance_scalars_work")
atm_advance_scalars_mono_work = _operator("atm_advance_scalars_mono_work")
mpas_reconstruct_2d = _operator("mpas_reconstruct_2d")

__all__ = ["use_mesh", "ROUTINES", *ROUTINES]
