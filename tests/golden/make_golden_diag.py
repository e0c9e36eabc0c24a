"""Golden vectors for the surface-pressure diagnostic, made by the reference itself.

Runs the reference's ``physics_interface_surface_pressure`` (mpas_pytorch/diagnostics.py:10)
on the evolved states stored in the committed ``g2_*`` fixtures (after step 1 and step 2)
and writes ``sp_g2.npz`` (one array per case and step).  Imports the reference the same
way as ``make_golden.py`` (netCDF4 stub).

Run:  python tests/golden/make_golden_diag.py
"""

from __future__ import annotations

import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent))

import make_golden  # noqa: E402
from fixtures import group, load_case  # noqa: E402


def main() -> None:
    make_golden._import_reference()
    import torch
    from mpas_pytorch.diagnostics import physics_interface_surface_pressure

    out = {}
    for case in ("g2_explicit", "g2_mono"):
        meta, st, _ = load_case(case)
        loaded, prepared = group(st, "loaded"), group(st, "prepared")
        nc = int(np.asarray(loaded["nCells"]).reshape(-1)[0])
        for step in ("step1", "step2"):
            s = group(st, step)
            t = lambda a: torch.as_tensor(np.asarray(a), dtype=torch.float64)
            sp = physics_interface_surface_pressure(
                nCells=nc, rho_zz=t(s["rho_zz"]), zz=t(loaded["zz"]), qv=t(s["scalars"][..., 0]),
                pressure_p=t(s["pressure_p"]), pressure_base=t(prepared["pressure_base"]),
                zgrid=t(loaded["zgrid"]))
            out[f"{case}/{step}"] = sp.numpy()
    np.savez_compressed(HERE / "sp_g2.npz", **out)
    print("wrote", HERE / "sp_g2.npz", sorted(out))


if __name__ == "__main__":
    main()
