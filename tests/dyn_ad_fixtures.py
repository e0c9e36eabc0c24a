"""Loader for the whole-step derivative fixtures made by tests/golden/make_golden_dyn_ad.py."""

from __future__ import annotations

import functools
import pathlib

import numpy as np

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
AD_CASES = ("g2_ad", "g2_ad_rk2")
# the mixing and damping options (vertical mixing, CAM and Rayleigh damping)
AD_OPTION_CASES = ("g2_ad_opts", "g2_ad_fixed")
# terrain-following levels over a cosine hill (the oracle's reverse sweep does not cover them)
AD_TERRAIN_CASES = ("g2_ad_terrain", "g2_ad_terrain_fixed")
BASE_CONFIG = {"config_time_integration_order": 3, "config_len_disp": 120000.0,
               "config_number_of_sub_steps": 2, "config_dynamics_split_steps": 3}
# the case options of make_golden_dyn_ad.CASES (kept here so the tests need no reference tree)
CASE_CONFIG = {
    "g2_ad": dict(config_monotonic=False),
    "g2_ad_rk2": dict(config_monotonic=False, config_time_integration_order=2, config_number_of_sub_steps=4,
                      config_dynamics_split_steps=2, config_horiz_mixing="2d_fixed",
                      config_h_mom_eddy_visc4=1.0e10, config_h_theta_eddy_visc4=5.0e9,
                      config_h_theta_eddy_visc2=2.0e4),
    "g2_ad_opts": dict(config_monotonic=False, config_mpas_cam_coef=1.0, config_number_cam_damping_levels=4,
                       config_rayleigh_damp_u=True, config_rayleigh_damp_u_timescale_days=0.5,
                       config_number_rayleigh_damp_u_levels=4, config_mix_full=False,
                       config_v_mom_eddy_visc2=2.0, config_v_theta_eddy_visc2=2.0),
    "g2_ad_fixed": dict(config_monotonic=False, config_horiz_mixing="2d_fixed", config_h_mom_eddy_visc4=1.0e10,
                        config_h_theta_eddy_visc4=5.0e9, config_h_theta_eddy_visc2=2.0e4,
                        config_mpas_cam_coef=1.0, config_number_cam_damping_levels=3,
                        config_v_mom_eddy_visc2=1.0, config_v_theta_eddy_visc2=1.0),
    "g2_ad_terrain": dict(config_monotonic=False),
    "g2_ad_terrain_fixed": dict(config_monotonic=False, config_horiz_mixing="2d_fixed",
                                config_h_mom_eddy_visc4=1.0e10, config_h_theta_eddy_visc4=5.0e9,
                                config_h_theta_eddy_visc2=2.0e4),
}
DIMS = ("nCells", "nEdges", "nVertices", "nVertLevels", "maxEdges", "maxEdges2", "vertexDegree")
LOADED_SCALARS = {"c_s": 0.125, "coef_3rd_order": 0.25, "moist_start": 1, "moist_end": 0}


@functools.lru_cache(maxsize=None)
def _npz(case):
    return dict(np.load(GOLDEN / f"dyn_ad_{case}.npz"))


def config(case):
    z = _npz(case)
    cfg = dict(BASE_CONFIG)
    cfg.update(CASE_CONFIG[case])
    cfg["config_dt"] = float(z["dt"])
    return cfg


def mesh_and_state(case):
    """(mesh, loaded state) as numpy mappings; dimensions as ints."""
    z = _npz(case)
    lo = {k[len("loaded/"):]: v for k, v in z.items() if k.startswith("loaded/")}
    mesh = dict(lo)
    mesh.update(LOADED_SCALARS)
    for k in DIMS:
        if k in mesh:
            mesh[k] = int(np.asarray(mesh[k]).reshape(-1)[0])
    return mesh, dict(lo)


def load_ad_case(case):
    from oracle.step import Stepper
    z = _npz(case)
    mesh, st0 = mesh_and_state(case)
    stepper = Stepper(mesh, config(case))
    return z, stepper, st0, float(z["dt"]), int(z["nsteps"])


def objective_cotangents(stepper, z, final):
    """J = sum area (sp - sp_ref)^2 of the final state (dry, qv = 0) and its cotangents of
    the final rho_zz and pressure_p (oracle restatements)."""
    import oracle.adjoint as A
    import oracle.stages as S
    m, nc = stepper.m, stepper.nc
    qv0 = np.zeros_like(final["rho_zz"])
    sp = S.surface_pressure(nc, final["rho_zz"], m["zz"], qv0, final["pressure_p"], final["pressure_base"],
                            m["zgrid"])[:nc]
    area = m["areaCell"][:nc]
    d = sp - z["sp_ref"]
    J = float((area * d * d).sum())
    g_sp = np.zeros(nc + 1)
    g_sp[:nc] = 2.0 * area * d
    gsp = A.surface_pressure_vjp(nc, final["rho_zz"], m["zz"], qv0, m["zgrid"], g_sp)
    return J, {"rho_zz": gsp["rho_zz"], "pressure_p": gsp["pressure_p"]}
