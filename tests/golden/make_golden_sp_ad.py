"""Golden derivatives of the surface-pressure diagnostic, made by the reference itself.

Runs the reference's ``physics_interface_surface_pressure`` (mpas_pytorch/diagnostics.py:10)
on the evolved state after step 2 of the committed ``g2_explicit`` and ``g2_moist``
fixtures (padded rows, qv = scalar 0, as ``make_golden_diag.py`` does) and records

* reverse mode: ``torch.autograd.grad`` of ``sum(g_sp * sp)`` with respect to ``rho_zz``,
  ``qv``, ``pressure_p`` and ``pressure_base`` for a seeded cotangent ``g_sp``;
* forward mode: ``torch.autograd.forward_ad`` tangent of ``sp`` for seeded tangents of the
  same four inputs;
* the area-weighted squared-anomaly objective ``sum(area * (sp - sp_ref)^2)`` over the
  active cells and its gradient with respect to ``sp`` (torch autograd on the reference's
  output, seeded ``sp_ref``).

Writes ``sp_ad_g2.npz``.  Imports the reference the same way as ``make_golden.py``
(netCDF4 stub).

Run:  MPAS_REFERENCE=<reference tree> python tests/golden/make_golden_sp_ad.py
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

CASES = ("g2_explicit", "g2_moist")
DIFF = ("rho_zz", "qv", "pressure_p", "pressure_base")


def main() -> None:
    make_golden._import_reference()
    import torch
    import torch.autograd.forward_ad as fwAD
    from mpas_pytorch.diagnostics import physics_interface_surface_pressure

    out = {}
    for ci, case in enumerate(CASES):
        _, st, _ = load_case(case)
        lo, pr, s = group(st, "loaded"), group(st, "prepared"), group(st, "step2")
        nc = int(np.asarray(lo["nCells"]).reshape(-1)[0])
        t = lambda a: torch.as_tensor(np.ascontiguousarray(np.asarray(a)), dtype=torch.float64)
        args = dict(rho_zz=t(s["rho_zz"]), zz=t(lo["zz"]), qv=t(s["scalars"][..., 0]),
                    pressure_p=t(s["pressure_p"]), pressure_base=t(pr["pressure_base"]), zgrid=t(lo["zgrid"]))
        rows, nlev = args["rho_zz"].shape
        rng = np.random.default_rng(700 + ci)
        g_sp = t(rng.standard_normal(rows))
        tangents = {k: t(rng.standard_normal((rows, nlev)) * (1e-3 if k == "qv" else 1.0)) for k in DIFF}
        sp_ref = t(rng.uniform(0.99, 1.01, nc)) * 1.0e5
        area = t(rng.uniform(0.5, 1.5, nc)) * 1.0e10

        # reverse mode
        leaf = {k: (v.clone().requires_grad_(True) if k in DIFF else v) for k, v in args.items()}
        sp = physics_interface_surface_pressure(nCells=nc, **leaf)
        grads = torch.autograd.grad((g_sp * sp).sum(), [leaf[k] for k in DIFF])
        # forward mode
        with fwAD.dual_level():
            dual = {k: (fwAD.make_dual(v, tangents[k]) if k in DIFF else v) for k, v in args.items()}
            sp_t = fwAD.unpack_dual(physics_interface_surface_pressure(nCells=nc, **dual)).tangent
        # objective and its gradient with respect to sp
        spl = sp.detach()[:nc].clone().requires_grad_(True)
        obj = (area * (spl - sp_ref) ** 2).sum()
        (g_obj,) = torch.autograd.grad(obj, [spl])

        out[f"{case}/nCells"] = np.array(nc)
        out[f"{case}/sp"] = sp.detach().numpy()
        out[f"{case}/g_sp"] = g_sp.numpy()
        for k, g in zip(DIFF, grads):
            out[f"{case}/grad_{k}"] = g.numpy()
            out[f"{case}/tan_{k}"] = tangents[k].numpy()
        out[f"{case}/sp_tangent"] = sp_t.numpy()
        out[f"{case}/sp_ref"] = sp_ref.numpy()
        out[f"{case}/area"] = area.numpy()
        out[f"{case}/objective"] = np.array(obj.item())
        out[f"{case}/grad_objective_sp"] = g_obj.numpy()
    np.savez_compressed(HERE / "sp_ad_g2.npz", **out)


if __name__ == "__main__":
    main()
