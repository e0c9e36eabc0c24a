"""The oracle's reverse sweep of whole large steps (oracle/dyn_adjoint.py) against the
gradients the reference itself computed (run_simulation.vjp of the area-weighted squared
surface-pressure anomaly with respect to the initial u and theta;
tests/golden/make_golden_dyn_ad.py)."""

import numpy as np
import pytest

from dyn_ad_fixtures import AD_CASES, AD_OPTION_CASES, AD_TERRAIN_CASES, load_ad_case, objective_cotangents
import oracle.dyn_adjoint as D


@pytest.mark.parametrize("case", AD_CASES + AD_OPTION_CASES + AD_TERRAIN_CASES)
def test_oracle_run_vjp_matches_reference(case):
    z, stepper, st0, dt, nsteps = load_ad_case(case)
    _, final = D.run_vjp(stepper, st0, dt, nsteps, {})
    J, g_final = objective_cotangents(stepper, z, final)
    assert abs(J - float(z["J"])) <= 1e-12 * float(z["J"])
    grads, _ = D.run_vjp(stepper, st0, dt, nsteps, g_final)
    for k in ("u", "theta"):
        a, b = grads[k][:-1], z[f"grad_{k}"][:-1]
        assert np.linalg.norm(a - b) <= 1e-11 * np.linalg.norm(b), k


@pytest.mark.parametrize("extra", [{"qtot": np.full((2, 4), 1e-3)}])
def test_oracle_stage_vjp_scope_is_enforced(extra):
    """Moist columns are refused, not silently mis-differentiated."""
    with pytest.raises(NotImplementedError):
        D.dyn_tend_vjp(dict({"nCells": 1, "nEdges": 1, "nVertices": 1, "nVertLevels": 4, "rk_step": 1,
                             "dt": 1.0, "coef_3rd_order": 0.25, "c_s": 0.125, "config_len_disp": 1.0,
                             "config_del4u_div_factor": 10.0, "config_horiz_mixing": "2d_fixed",
                             "config_h_mom_eddy_visc4": 0.0, "config_h_theta_eddy_visc4": 0.0}, **extra), {})
