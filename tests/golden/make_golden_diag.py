"""Golden vectors for the surface-pressure diagnostic and the RCM reordering, made by
the reference itself.

Runs the reference's ``physics_interface_surface_pressure`` (mpas_pytorch/diagnostics.py:10)
on the evolved states stored in the committed ``g2_*`` fixtures (after step 1 and step 2)
and writes ``sp_g2.npz`` (one array per case and step); runs ``apply_rcm_reordering``
(mpas_pytorch/mesh_reordering.py:243) on the ``g2_explicit`` loaded mesh and writes the
permutations and the reordered connectivity / fields to ``rcm_g2.npz``; runs the
reference's ``TridiagonalSolve`` and ``TridiagonalFactorize`` (forward, reverse mode
through ``torch.autograd.grad``, forward mode through ``torch.autograd.forward_ad``) on
seeded diagonally dominant column systems and writes ``tridiag_ref.npz``.  Imports the
reference the same way as ``make_golden.py`` (netCDF4 stub).

Also runs the reference's ``run_simulation.vjp`` / ``.jvp`` with respect to the scalars on
the g2_explicit case (two steps) and writes the weights, tangent and results to
``scalars_ad_g2.npz``; the same in the coupled transport mode (g2_coupled mesh, explicit
stages) to ``scalars_ad_g2_coupled.npz``.

Run:  MPAS_REFERENCE=<reference tree> python tests/golden/make_golden_diag.py
"""

from __future__ import annotations

import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent))

import make_golden  # noqa: E402
from fixtures import CASES, group, load_case  # noqa: E402


def main() -> None:
    mp = make_golden._import_reference()
    import torch
    from mpas_pytorch.diagnostics import physics_interface_surface_pressure

    out = {}
    for case in CASES:
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

    # the reference's own JVP / VJP of run_simulation with respect to the scalars
    # (atmosphere_model.py:2041, :2101) on g2_explicit (explicit transport, passive tracer),
    # two steps: objective = sum(weights * final scalars), seeded weights and tangent
    ad = {}
    state, meshd, cfg = make_golden.load_reference_case(mp, make_golden.CASES["g2_explicit"])
    g = torch.Generator().manual_seed(20261203)
    sc = state["scalars"]
    wts = torch.rand(sc.shape, generator=g, dtype=torch.float64)
    tan = torch.randn(sc.shape, generator=g, dtype=torch.float64)
    kw = dict(config=cfg, dt=make_golden.CASES["g2_explicit"]["dt"], nsteps=2)
    grads = mp.run_simulation.vjp(state, meshd, lambda o: (o["scalars"] * wts).sum(), track_keys=("scalars",), **kw)
    tangents = mp.run_simulation.jvp(state, meshd, {"scalars": tan}, **kw)
    ad.update({"weights": wts.numpy(), "vjp_scalars": grads["scalars"].detach().numpy(),
               "tangent": tan.numpy(), "jvp_scalars": tangents["scalars"].detach().numpy(),
               "jvp_keys": np.array(sorted(tangents))})
    np.savez_compressed(HERE / "scalars_ad_g2.npz", **ad)
    print("wrote", HERE / "scalars_ad_g2.npz", sorted(ad))

    # the same in the coupled transport mode (config_split_dynamics_transport = false: the
    # scalars advance inside every RK stage with that stage's fluxes), explicit stages,
    # on the g2_coupled mesh and tracers, two steps
    case = dict(make_golden.CASES["g2_coupled"], config=dict(config_monotonic=False,
                                                             config_split_dynamics_transport=False))
    state, meshd, cfg = make_golden.load_reference_case(mp, case)
    g = torch.Generator().manual_seed(20261204)
    sc = state["scalars"]
    wts = torch.rand(sc.shape, generator=g, dtype=torch.float64)
    tan = torch.randn(sc.shape, generator=g, dtype=torch.float64)
    kw = dict(config=cfg, dt=case["dt"], nsteps=2)
    grads = mp.run_simulation.vjp(state, meshd, lambda o: (o["scalars"] * wts).sum(), track_keys=("scalars",), **kw)
    tangents = mp.run_simulation.jvp(state, meshd, {"scalars": tan}, **kw)
    adc = {"weights": wts.numpy(), "vjp_scalars": grads["scalars"].detach().numpy(), "tangent": tan.numpy(),
           "jvp_scalars": tangents["scalars"].detach().numpy(), "config": np.array(repr(cfg)),
           "dt": np.array(case["dt"])}
    np.savez_compressed(HERE / "scalars_ad_g2_coupled.npz", **adc)
    print("wrote", HERE / "scalars_ad_g2_coupled.npz", sorted(adc))
    print("wrote", HERE / "sp_g2.npz", sorted(out))

    from mpas_pytorch.mesh_reordering import apply_rcm_reordering
    meta, st, _ = load_case("g2_explicit")
    loaded = group(st, "loaded")
    mesh = {k: (torch.as_tensor(np.asarray(v)) if np.ndim(v) > 0 else int(np.asarray(v)) if np.asarray(v).dtype.kind in "iu"
                else float(np.asarray(v))) for k, v in loaded.items()}
    state = {k: mesh[k] for k in ("u", "theta", "rho", "w", "scalars")}
    rst, rmesh = apply_rcm_reordering(state, mesh)
    rec = {f"perm/{k}": v.numpy() for k, v in rmesh["_rcm_permutation"].items()}
    for k in ("cellsOnEdge", "edgesOnCell", "cellsOnCell", "verticesOnEdge", "edgesOnEdge", "advCellsForEdge",
              "edgesOnVertex", "cellsOnVertex", "verticesOnCell", "kiteForCell", "dvEdge", "areaCell", "weightsOnEdge"):
        rec[f"mesh/{k}"] = rmesh[k].numpy()
    for k in ("u", "theta", "w", "scalars"):
        rec[f"state/{k}"] = rst[k].numpy()
    np.savez_compressed(HERE / "rcm_g2.npz", **rec)
    print("wrote", HERE / "rcm_g2.npz", len(rec))

    import torch.autograd.forward_ad as fw
    from mpas_pytorch.autodiff.tridiagonal_factor import TridiagonalFactorize
    from mpas_pytorch.autodiff.tridiagonal_solve import TridiagonalSolve
    rec = {}
    for n, L in ((3, 6), (17, 41)):
        g = torch.Generator().manual_seed(1000 * n + L)
        r = lambda *s: torch.randn(*s, generator=g, dtype=torch.float64)
        a, c = 0.1 * r(n, L), 0.1 * r(n, L)
        b = 1.0 + 0.1 * torch.rand(n, L, generator=g, dtype=torch.float64)
        al, ga = TridiagonalFactorize.apply(a, b, c)
        rhs = r(n, L + 1)
        out = TridiagonalSolve.apply(a, al, ga, rhs)
        tag = f"{n}x{L}"
        rec.update({f"{tag}/a": a.numpy(), f"{tag}/b": b.numpy(), f"{tag}/c": c.numpy(), f"{tag}/rhs": rhs.numpy(),
                    f"{tag}/alpha": al.numpy(), f"{tag}/gamma": ga.numpy(), f"{tag}/out": out.numpy()})
        w, wa, wg = r(n, L + 1), r(n, L), r(n, L)
        ins = [t.clone().requires_grad_(True) for t in (a, al, ga, rhs)]
        o = TridiagonalSolve.apply(*ins)
        grads = torch.autograd.grad((o * w).sum(), ins)
        for nm, gr in zip(("a", "alpha", "gamma", "rhs"), grads):
            rec[f"{tag}/solve_vjp_{nm}"] = gr.numpy()
        rec[f"{tag}/solve_w"] = w.numpy()
        tans = [r(*t.shape) for t in (a, al, ga, rhs)]
        with fw.dual_level():
            duals = [fw.make_dual(p, t) for p, t in zip((a, al, ga, rhs), tans)]
            _, tout = fw.unpack_dual(TridiagonalSolve.apply(*duals))
        for nm, t in zip(("a", "alpha", "gamma", "rhs"), tans):
            rec[f"{tag}/solve_tan_{nm}"] = t.numpy()
        rec[f"{tag}/solve_jvp"] = tout.numpy()
        fins = [t.clone().requires_grad_(True) for t in (a, b, c)]
        fal, fga = TridiagonalFactorize.apply(*fins)
        fgrads = torch.autograd.grad((fal * wa).sum() + (fga * wg).sum(), fins)
        rec[f"{tag}/factor_wa"], rec[f"{tag}/factor_wg"] = wa.numpy(), wg.numpy()
        for nm, gr in zip(("a", "b", "c"), fgrads):
            rec[f"{tag}/factor_vjp_{nm}"] = gr.numpy()
        ftans = [r(n, L) for _ in range(3)]
        with fw.dual_level():
            duals = [fw.make_dual(p, t) for p, t in zip((a, b, c), ftans)]
            o1, o2 = TridiagonalFactorize.apply(*duals)
            rec[f"{tag}/factor_jvp_alpha"] = fw.unpack_dual(o1)[1].numpy()
            rec[f"{tag}/factor_jvp_gamma"] = fw.unpack_dual(o2)[1].numpy()
        for nm, t in zip(("a", "b", "c"), ftans):
            rec[f"{tag}/factor_tan_{nm}"] = t.numpy()
    np.savez_compressed(HERE / "tridiag_ref.npz", **rec)
    print("wrote", HERE / "tridiag_ref.npz", len(rec))


if __name__ == "__main__":
    main()
