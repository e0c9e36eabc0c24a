"""Golden continuations of a returned step boundary, made by the reference itself.

The reference binds the boundary ``run_simulation`` returns (state.py:194
``mark_complete_step_boundary``); a later call continues from a bound boundary as it is,
re-derives the coupled diagnostics of one whose prognostics were edited
(atmosphere_model.py:829-898), and rejects one whose diagnostics were edited or that
continues with another time step.  On the g2_explicit case (level-2 mesh, 162 cells x 12
levels, dt 1800 s) this records:

* ``cont/*``: one step, then one more from the returned boundary (equal, bit for bit, to
  two steps in one call);
* ``edit/*``: one step, then one more from the returned boundary with theta_m[5, 3]
  scaled by 1.0001 and u[7, 2] raised by 0.5 m/s (re-derived before the step);
* the reference's messages for an edited diagnostic (exner) and for another time step.

Writes ``boundary_g2_explicit.npz`` and ``boundary_g2_explicit.json``.  Imports the
reference the same way as ``make_golden.py`` (netCDF4 stub).

Run:  MPAS_REFERENCE=<reference tree> python tests/golden/make_golden_boundary.py
"""

from __future__ import annotations

import copy
import json
import os
import pathlib
import sys

import numpy as np

os.environ["PYTHONDONTWRITEBYTECODE"] = "1"
os.environ.setdefault("ATEN_CPU_CAPABILITY", "default")

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent))

import make_golden  # noqa: E402

CASE = "g2_explicit"
KEYS = ("u", "w", "theta_m", "rho_zz", "scalars", "pressure_p", "exner", "rho_p", "rtheta_p", "ru", "rw", "v",
        "divergence", "vorticity", "ke", "pv_edge", "h_edge")
EDIT_THETA = (5, 3, 1.0001)   # theta_m[5, 3] *= 1.0001
EDIT_U = (7, 2, 0.5)          # u[7, 2] += 0.5


def main() -> None:
    import torch
    mp = make_golden._import_reference()
    case = make_golden.CASES[CASE]
    state, mesh, cfg = make_golden.load_reference_case(mp, case)
    dt = case["dt"]

    def clone(d):
        return {k: (v.clone() if isinstance(v, torch.Tensor) else copy.deepcopy(v)) for k, v in d.items()}

    b1 = mp.run_simulation(state, mesh, config=cfg, dt=dt, nsteps=1)
    edited, diag_edit, dt_edit = clone(b1), clone(b1), clone(b1)
    cont = mp.run_simulation(b1, mesh, config=cfg, dt=dt, nsteps=1)
    edited["theta_m"] = edited["theta_m"].clone()
    edited["theta_m"][EDIT_THETA[0], EDIT_THETA[1]] *= EDIT_THETA[2]
    edited["u"] = edited["u"].clone()
    edited["u"][EDIT_U[0], EDIT_U[1]] += EDIT_U[2]
    edit = mp.run_simulation(edited, mesh, config=cfg, dt=dt, nsteps=1)
    messages = {}
    diag_edit["exner"] = diag_edit["exner"].clone()
    diag_edit["exner"][5, 3] *= 1.0001
    for label, st, step in (("diagnostic_edit", diag_edit, dt), ("other_dt", dt_edit, dt / 2)):
        try:
            mp.run_simulation(st, mesh, config=cfg, dt=step, nsteps=1)
            messages[label] = None
        except Exception as exc:  # noqa: BLE001 - the reference's message is the record
            messages[label] = f"{type(exc).__name__}: {exc}"
    out = {}
    for tag, st in (("cont", cont), ("edit", edit)):
        for k in KEYS:
            out[f"{tag}/{k}"] = st[k].detach().numpy().copy()
    np.savez_compressed(HERE / f"boundary_{CASE}.npz", **out)
    meta = {"case": CASE, "dt": dt, "edit_theta_m": EDIT_THETA, "edit_u": EDIT_U, "messages": messages,
            "torch": torch.__version__}
    (HERE / f"boundary_{CASE}.json").write_text(json.dumps(meta, indent=1))
    print(json.dumps(meta, indent=1))


if __name__ == "__main__":
    main()
