"""Every public route rejects unsupported requests before any preparation or device work
(the reference's contract, tests/test_configuration_contracts.py of mpas_pytorch): active
physics / assimilation / restart / regional / sharding settings, and reduced-precision
float storage.  Runs on CPU: nothing here may reach the device."""

import pytest
import torch

import mpas_dycore_pytorch_gb300 as gb
from mpas_dycore_pytorch_gb300.api import active_unsupported_settings
from mpas_dycore_pytorch_gb300.errors import MpasConfigError, MpasUnsupportedCapabilityError

UNSUPPORTED = [
    ("config_physics_suite", "mesoscale_reference"),
    ("config_microp_scheme", "mp_wsm6"),
    ("config_IAU_option", "incremental"),
    ("config_do_DAcycling", True),
    ("config_jedi_da", "true"),
    ("config_jedi_da", ".true."),
    ("config_apply_lbcs", True),
    ("config_enable_sharding", True),
    ("config_enable_sharding", ".true."),
    ("config_explicit_proc_decomp", True),
    ("config_do_restart", "T"),
]


def _call(route, state, mesh, config):
    kw = {"config": config, "dt": 720.0}
    if route == "timestep":
        return gb.run_timestep(state, mesh, **kw)
    if route == "simulation":
        return gb.run_simulation(state, mesh, nsteps=1, **kw)
    if route == "jvp":
        return gb.run_simulation.jvp(state, mesh, {"u": torch.zeros_like(state["u"])}, nsteps=1, **kw)
    return gb.run_simulation.vjp(state, mesh, lambda out: out["u"].sum(), track_keys=["u"], nsteps=1, **kw)


@pytest.mark.parametrize("route", ["timestep", "simulation", "jvp", "vjp"])
@pytest.mark.parametrize("key,value", UNSUPPORTED)
def test_unsupported_configuration_rejected_first(route, key, value):
    # a state no preparation could use: only an up-front rejection can raise this error
    state = {"u": torch.ones((2, 1), dtype=torch.float64)}
    with pytest.raises(MpasUnsupportedCapabilityError):
        _call(route, state, {}, {key: value})


@pytest.mark.parametrize("route", ["timestep", "simulation", "jvp", "vjp"])
@pytest.mark.parametrize("location", ["state", "mesh"])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float16, torch.bfloat16])
def test_reduced_precision_storage_rejected_first(route, location, dtype):
    state = {"u": torch.ones((2, 1), dtype=torch.float64)}
    mesh = {"dcEdge": torch.ones(2, dtype=torch.float64)}
    target, key = (state, "u") if location == "state" else (mesh, "dcEdge")
    target[key] = target[key].to(dtype)
    with pytest.raises(MpasUnsupportedCapabilityError, match="dtype"):
        _call(route, state, mesh, {})


def test_inactive_values_pass():
    cfg = {"config_physics_suite": "none", "config_IAU_option": "off", "config_jedi_da": ".false.",
           "config_apply_lbcs": "F", "config_enable_sharding": 0, "config_microp_scheme": "off"}
    assert active_unsupported_settings(cfg) == []


def test_ambiguous_logical_is_a_config_error():
    with pytest.raises(MpasConfigError):
        active_unsupported_settings({"config_jedi_da": "maybe"})


@pytest.mark.parametrize("key", ["u", "theta", "scalars"])
def test_nonfinite_inputs_rejected_first(key):
    state = {"u": torch.ones((2, 1), dtype=torch.float64), "theta": torch.ones((2, 1), dtype=torch.float64),
             "scalars": torch.ones((2, 1, 1), dtype=torch.float64)}
    state[key][0] = float("nan")
    with pytest.raises(MpasConfigError, match="nonfinite"):
        gb.run_simulation(state, {}, config={}, nsteps=1)
