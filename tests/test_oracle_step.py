"""Oracle preparation and full large steps against the reference's boundaries."""

import numpy as np
import pytest

from oracle.step import Stepper
from fixtures import CASES, group, load_case, rel_l2, step_tol

FIELDS = ("u", "w", "theta_m", "rho_zz", "scalars", "rho_p", "rtheta_p", "exner", "pressure_p",
          "ru", "rw", "v", "divergence", "vorticity", "ke", "pv_edge", "rho_edge",
          "uReconstructX", "uReconstructY", "uReconstructZ", "uReconstructZonal",
          "uReconstructMeridional", "ruAvg", "wwAvg")


def _setup(case):
    meta, st, _ = load_case(case)
    loaded = group(st, "loaded")
    mesh = dict(loaded)
    mesh.update(meta["loaded_scalars"])
    return meta, st, loaded, Stepper(mesh, meta["config"])


@pytest.mark.parametrize("case", CASES)
def test_prepare_matches_reference(case):
    meta, st, loaded, stepper = _setup(case)
    prep = stepper.prepare(loaded, meta["dt"])
    ref = group(st, "prepared")
    for k in ("theta_m", "rho_zz", "ru", "rw", "rho_p", "rtheta_p", "exner", "v", "vorticity",
              "divergence", "ke", "pv_edge", "rho_edge", "uReconstructZonal",
              "uReconstructMeridional", "pressure_p"):
        assert rel_l2(prep[k][:-1], ref[k][:-1]) <= 1e-15, k


@pytest.mark.parametrize("case", CASES)
def test_two_steps_match_reference(case):
    meta, st, _, stepper = _setup(case)
    state = group(st, "prepared")
    for step in (1, 2):
        state = stepper.srk3_step(state, meta["dt"])
        ref = group(st, f"step{step}")
        for k in FIELDS:
            assert rel_l2(state[k][:-1], ref[k][:-1]) <= step_tol(case, k), (step, k)
        assert np.array_equal(state["scalars"][-1], ref["scalars"][-1])
