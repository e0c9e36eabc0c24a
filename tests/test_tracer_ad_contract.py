"""Argument contract of run_simulation.vjp / .jvp on the GB300 path (CPU: everything
here is rejected before any device work)."""

import numpy as np
import pytest
import torch

from mpas_dycore_pytorch_gb300.api import run_simulation
from mpas_dycore_pytorch_gb300.errors import MpasConfigError, MpasUnsupportedCapabilityError
from fixtures import group, load_case


def _case():
    meta, st, _ = load_case("g2_explicit")
    state = {k: torch.as_tensor(v) for k, v in group(st, "loaded").items()}
    state.update(meta["loaded_scalars"])
    return state, meta


def test_vjp_track_keys_contract():
    """The scalars, or the dynamics keys u / w / theta / rho, never both; nothing else."""
    state, meta = _case()
    for keys in (None, ("scalars", "theta"), ("theta_m",)):
        with pytest.raises(MpasUnsupportedCapabilityError):
            run_simulation.vjp(state, state, lambda o: o["scalars"].sum(), track_keys=keys, config=meta["config"])


@pytest.mark.parametrize("extra", [{"config_v_mom_eddy_visc2": 1.0}, {"config_v_theta_eddy_visc2": 1.0},
                                   {"config_mpas_cam_coef": 1.0}, {"config_rayleigh_damp_u": True},
                                   {"config_mix_full": False, "config_v_mom_eddy_visc2": 1.0}])
def test_dynamics_derivative_scope_takes_the_mixing_and_damping_options(extra):
    """Vertical mixing, CAM and Rayleigh damping are differentiated, over terrain too: the
    host-side scope check passes them (moisture is what it still refuses)."""
    from mpas_dycore_pytorch_gb300.dyn_adjoint import check_request
    state, meta = _case()
    cfg = dict(meta["config"], **extra)
    n = int(state["scalars"].shape[-1])
    check_request(cfg, state, n)
    check_request(cfg, dict(state, zb_cell=np.ones((3, 2))), n)
    with pytest.raises(MpasUnsupportedCapabilityError, match="dry columns"):
        check_request(cfg, dict(state, moist_start=0, moist_end=0), n)


def test_dynamics_jvp_is_float64_only():
    """The reverse mode takes the mixed form; the forward mode is float64 only."""
    state, meta = _case()
    cfg = dict(meta["config"], config_precision="mixed")
    with pytest.raises(MpasUnsupportedCapabilityError, match="float64"):
        run_simulation.jvp(state, state, {"u": torch.zeros_like(state["u"])}, config=cfg)


def test_dynamics_vjp_moist_rejected_before_device_work():
    state, meta = _case()
    state = dict(state, moist_end=1)
    with pytest.raises(MpasUnsupportedCapabilityError):
        run_simulation.vjp(state, state, lambda o: o["rho_zz"].sum(), track_keys=("theta",), config=meta["config"])


@pytest.mark.parametrize("extra", [{"config_monotonic": True}, {"config_positive_definite": True},
                                   {"config_monotonic": True, "config_split_dynamics_transport": False},
                                   {"config_scalar_advection": False}])
def test_unsupported_transport_rejected(extra):
    state, meta = _case()
    cfg = dict(meta["config"], **extra)
    with pytest.raises(MpasUnsupportedCapabilityError):
        run_simulation.vjp(state, state, lambda o: o["scalars"].sum(), track_keys=("scalars",), config=cfg)
    with pytest.raises(MpasUnsupportedCapabilityError):
        run_simulation.jvp(state, state, {"scalars": torch.zeros_like(state["scalars"])}, config=cfg)


def test_moist_scalars_rejected():
    state, meta = _case()
    state = dict(state, moist_end=1)
    with pytest.raises(MpasUnsupportedCapabilityError):
        run_simulation.vjp(state, state, lambda o: o["scalars"].sum(), track_keys=("scalars",), config=meta["config"])


def test_jvp_perturbation_contract():
    state, meta = _case()
    # the dynamics tangents cover dry columns only
    moist = dict(state, moist_end=1)
    with pytest.raises(MpasUnsupportedCapabilityError, match="dry columns"):
        run_simulation.jvp(moist, moist, {"u": torch.zeros_like(state["u"])}, config=meta["config"])
    with pytest.raises(MpasUnsupportedCapabilityError, match="not both kinds"):
        run_simulation.jvp(state, state, {"u": torch.zeros_like(state["u"]),
                                          "scalars": torch.zeros_like(state["scalars"])}, config=meta["config"])
    with pytest.raises(KeyError):
        run_simulation.jvp(state, state, {"theta_m": torch.zeros_like(state["u"])}, config=meta["config"])
    with pytest.raises(MpasConfigError):
        run_simulation.jvp(state, state, {"u": torch.zeros_like(state["u"], dtype=torch.float32)},
                           config=meta["config"])
    with pytest.raises(MpasConfigError):
        run_simulation.jvp(state, state, {"scalars": torch.zeros(3, 2)}, config=meta["config"])
    with pytest.raises(TypeError):
        run_simulation.jvp(state, state, {"scalars": np.zeros(3)}, config=meta["config"])


def test_differentiable_runs_take_scalars_or_the_dynamics_inputs():
    """differentiable=True carries gradients for the scalars or for the loaded u, w, theta,
    rho, not both; any other input requiring grad, and a dynamics input of a moist run,
    are rejected before any device work."""
    import mpas_dycore_pytorch_gb300 as gb
    from fixtures import group, load_case
    meta, st, _ = load_case("g2_explicit")
    state = {k: torch.as_tensor(v) for k, v in group(st, "loaded").items()}
    both = dict(state, u=state["u"].clone().requires_grad_(True),
                scalars=state["scalars"].clone().requires_grad_(True))
    with pytest.raises(gb.MpasUnsupportedCapabilityError, match="not both"):
        gb.run_simulation(both, state, meta["config"], meta["dt"], nsteps=1, differentiable=True)
    other = dict(state, zgrid=state["zgrid"].clone().requires_grad_(True))
    with pytest.raises(gb.MpasUnsupportedCapabilityError, match="zgrid"):
        gb.run_simulation(other, state, meta["config"], meta["dt"], nsteps=1, differentiable=True)
    moist = dict(state, u=state["u"].clone().requires_grad_(True), moist_end=1)
    with pytest.raises(gb.MpasUnsupportedCapabilityError, match="dry columns"):
        gb.run_simulation(moist, state, meta["config"], meta["dt"], nsteps=1, differentiable=True)