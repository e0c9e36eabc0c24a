"""Golden derivatives of whole large steps with respect to the initial wind and potential
temperature, made by the reference itself.

The differentiation workload's recipe on the level-2 mesh (162 cells x 12 levels): the
analytic dry state with a 0.1 m/s sinusoidal w and the wind rounded to 16 significant
bits (``CaseSpec(w_sine=0.1, round_wind_bits=16)``), RK3 with 3 dynamics substeps x 2
acoustic substeps, one passive tracer, dt 900 s.  The functional is the area-weighted
squared anomaly of the hydrostatic surface pressure at the final time,

    J = sum_c areaCell_c (sp_c(T) - sp_ref_c)^2,

``sp`` = ``physics_interface_surface_pressure`` (mpas_pytorch/diagnostics.py:10) of the
final ``rho_zz`` and ``pressure_p`` (dry: qv = 0), ``sp_ref`` the surface pressure of the
prepared initial state (a constant).  Recorded per case:

* ``run_simulation.vjp`` (atmosphere_model.py:2101) of J with ``track_keys=("u",
  "theta")``: the gradients ``grad_u`` and ``grad_theta``;
* ``run_simulation.jvp`` (atmosphere_model.py:2041) in a seeded direction (``dir_u``,
  ``dir_theta``; padding rows zero): the tangents of the final ``rho_zz``,
  ``pressure_p``, ``u``, ``theta_m`` and ``w``;
* the loaded state (``loaded/*``, the inputs), J and ``sp_ref``.

Writes ``dyn_ad_<case>.npz``.  Imports the reference the same way as ``make_golden.py``
(netCDF4 stub).

Run:  MPAS_REFERENCE=<reference tree> python tests/golden/make_golden_dyn_ad.py [case ...]
"""

from __future__ import annotations

import os
import pathlib
import sys
import time

import numpy as np

os.environ["PYTHONDONTWRITEBYTECODE"] = "1"
os.environ.setdefault("ATEN_CPU_CAPABILITY", "default")

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent))

import make_golden  # noqa: E402

CASES = {
    # two steps of the differentiation recipe
    "g2_ad": dict(spec=dict(level=2, nlev=12, seed=2, n_bumps=6, n_tracers=1, w_sine=0.1, round_wind_bits=16),
                  config=dict(config_monotonic=False), dt=900.0, nsteps=2),
    # RK2, four acoustic substeps, two dynamics substeps, fixed-coefficient mixing
    "g2_ad_rk2": dict(spec=dict(level=2, nlev=12, seed=12, n_bumps=6, n_tracers=1, w_sine=0.1,
                                round_wind_bits=16),
                      config=dict(config_monotonic=False, config_time_integration_order=2,
                                  config_number_of_sub_steps=4, config_dynamics_split_steps=2,
                                  config_horiz_mixing="2d_fixed", config_h_mom_eddy_visc4=1.0e10,
                                  config_h_theta_eddy_visc4=5.0e9, config_h_theta_eddy_visc2=2.0e4),
                      dt=900.0, nsteps=2),
    # the damping and mixing options: Smagorinsky mixing with CAM-style top-level damping,
    # Rayleigh damping of u, vertical mixing of the perturbation from nonzero initial profiles
    # (config_mix_full = false), stretched levels
    "g2_ad_opts": dict(spec=dict(level=2, nlev=12, dz_bottom=400.0, seed=13, n_bumps=6, n_tracers=1, w_sine=0.1,
                                 round_wind_bits=16, uv_init=(15.0, 2.0)),
                       config=dict(config_monotonic=False, config_mpas_cam_coef=1.0,
                                   config_number_cam_damping_levels=4, config_rayleigh_damp_u=True,
                                   config_rayleigh_damp_u_timescale_days=0.5,
                                   config_number_rayleigh_damp_u_levels=4, config_mix_full=False,
                                   config_v_mom_eddy_visc2=2.0, config_v_theta_eddy_visc2=2.0),
                       dt=900.0, nsteps=2),
    # fixed-coefficient mixing with CAM damping of the constant coefficient and vertical
    # mixing of the full state
    "g2_ad_fixed": dict(spec=dict(level=2, nlev=12, seed=14, n_bumps=6, n_tracers=1, w_sine=0.1,
                                  round_wind_bits=16),
                        config=dict(config_monotonic=False, config_horiz_mixing="2d_fixed",
                                    config_h_mom_eddy_visc4=1.0e10, config_h_theta_eddy_visc4=5.0e9,
                                    config_h_theta_eddy_visc2=2.0e4, config_mpas_cam_coef=1.0,
                                    config_number_cam_damping_levels=3, config_v_mom_eddy_visc2=1.0,
                                    config_v_theta_eddy_visc2=1.0),
                        dt=900.0, nsteps=2),
    # terrain-following levels over a 1500 m cosine hill (zz != 1, slope terms zb / zb3 / zxu)
    "g2_ad_terrain": dict(spec=dict(level=2, nlev=12, dz_bottom=400.0, seed=16, n_bumps=6, n_tracers=1,
                                    w_sine=0.1, round_wind_bits=16, terrain=1500.0),
                          config=dict(config_monotonic=False), dt=900.0, nsteps=2),
    # the same over fixed-coefficient del2 / del4 mixing (no Smagorinsky coefficient, whose
    # square root of a near-zero deformation makes the u gradient follow the roundings)
    "g2_ad_terrain_fixed": dict(spec=dict(level=2, nlev=12, dz_bottom=400.0, seed=17, n_bumps=6, n_tracers=1,
                                          w_sine=0.1, round_wind_bits=16, terrain=1500.0),
                                config=dict(config_monotonic=False, config_horiz_mixing="2d_fixed",
                                            config_h_mom_eddy_visc4=1.0e10, config_h_theta_eddy_visc4=5.0e9,
                                            config_h_theta_eddy_visc2=2.0e4),
                                dt=900.0, nsteps=2),
}
TRACK = ("u", "theta")
JVP_KEYS = ("rho_zz", "pressure_p", "u", "theta_m", "w")


def objective_factory(mp, mesh, sp_ref):
    import torch
    from mpas_pytorch.diagnostics import physics_interface_surface_pressure
    nc = int(mesh["nCells"])
    area = mesh["areaCell"][:nc]

    def surface_pressure(state):
        rz = state["rho_zz"]
        get = lambda k: state[k] if k in state else mesh[k]
        return physics_interface_surface_pressure(
            nCells=nc, rho_zz=rz, zz=get("zz"), qv=torch.zeros_like(rz),
            pressure_p=state["pressure_p"], pressure_base=get("pressure_base"), zgrid=get("zgrid"))

    def objective(state):
        sp = surface_pressure(state)[:nc]
        return (area * (sp - sp_ref) ** 2).sum()

    return surface_pressure, objective


def run_case(mp, name: str, case: dict) -> None:
    import torch
    state, meshd, cfg = make_golden.load_reference_case(mp, case)
    dt, nsteps = case["dt"], case["nsteps"]
    out: dict[str, np.ndarray] = {}
    for k, v in state.items():
        if isinstance(v, torch.Tensor):
            out[f"loaded/{k}"] = v.detach().numpy().copy()
    def fresh():
        # every run gets its own loaded state and mesh (a run rewrites the mesh mapping in place)
        return make_golden.load_reference_case(mp, case)[:2]

    prepared = {}
    st_, me_ = fresh()
    mp.run_simulation(st_, me_, config=cfg, dt=dt, nsteps=1,
                      on_initial=lambda s: prepared.update({k: v.detach().clone() for k, v in s.items()
                                                           if isinstance(v, torch.Tensor)}))
    sp_fn, _ = objective_factory(mp, meshd, None)
    nc = int(meshd["nCells"])
    sp_ref = sp_fn({**{k: v.clone() for k, v in prepared.items()}})[:nc].detach().clone()
    st_, me_ = fresh()
    _, objective = objective_factory(mp, me_, sp_ref)
    t0 = time.time()
    grads = mp.run_simulation.vjp(st_, me_, objective, track_keys=TRACK, config=cfg, dt=dt, nsteps=nsteps)
    t_vjp = time.time() - t0
    st_, me_ = fresh()
    final = mp.run_simulation(st_, me_, config=cfg, dt=dt, nsteps=nsteps)
    final = {k: (v.clone() if isinstance(v, torch.Tensor) else v) for k, v in final.items()}
    _, objective = objective_factory(mp, {k: (v.clone() if isinstance(v, torch.Tensor) else v)
                                          for k, v in me_.items()}, sp_ref)
    J = float(objective(final))
    rng = np.random.default_rng(20261204)
    direction = {}
    for k in TRACK:
        d = rng.standard_normal(tuple(state[k].shape))
        d[-1] = 0.0  # padding row: not perturbed (docs/API.md:118-119)
        direction[k] = torch.from_numpy(d * (1.0 if k == "u" else 0.1))
    t0 = time.time()
    st_, me_ = fresh()
    tang = mp.run_simulation.jvp(st_, me_, direction, config=cfg, dt=dt, nsteps=nsteps)
    t_jvp = time.time() - t0
    for k in TRACK:
        out[f"grad_{k}"] = grads[k].detach().numpy()
        out[f"dir_{k}"] = direction[k].numpy()
    for k in JVP_KEYS:
        out[f"jvp_{k}"] = tang[k].detach().numpy()
    out["J"] = np.array(J)
    out["sp_ref"] = sp_ref.numpy()
    out["dt"] = np.array(dt)
    out["nsteps"] = np.array(nsteps)
    np.savez_compressed(HERE / f"dyn_ad_{name}.npz", **out)
    print(f"{name}: J = {J:.6e}, vjp {t_vjp:.1f} s, jvp {t_jvp:.1f} s")


def main() -> None:
    mp = make_golden._import_reference()
    for name in sys.argv[1:] or list(CASES):
        run_case(mp, name, CASES[name])


if __name__ == "__main__":
    main()
