"""The reference's public names resolve here; the namelist and initial-state loaders
behave as the reference's; the netCDF I/O names fail with the typed error."""

import numpy as np
import pytest
import torch

import mpas_dycore_pytorch_gb300 as gb
from fixtures import group, load_case

REFERENCE_NAMES = {
    "MpasConfigError", "MpasDeviceError", "MpasError", "MpasMeshMismatchError", "MpasMissingFieldError",
    "MpasNumericalAgreementError", "MpasProvenanceError", "MpasStrictModeError", "MpasUnsupportedCapabilityError",
    "load_config_from_namelist", "load_initial_state", "read_history", "read_restart", "run_simulation",
    "run_timestep", "write_history", "write_restart",
}


def test_reference_surface_resolves():
    assert REFERENCE_NAMES <= set(gb.__all__)
    assert all(hasattr(gb, n) for n in REFERENCE_NAMES)
    assert callable(gb.run_simulation.jvp) and callable(gb.run_simulation.vjp)
    # the reference's hierarchy: configuration-side errors are MpasConfigError (ValueError)
    for n in ("MpasDeviceError", "MpasUnsupportedCapabilityError", "MpasMissingFieldError",
              "MpasMeshMismatchError", "MpasStrictModeError", "MpasProvenanceError"):
        assert issubclass(getattr(gb, n), gb.MpasConfigError)
    assert issubclass(gb.MpasConfigError, ValueError)
    assert issubclass(gb.MpasNumericalAgreementError, gb.MpasError)


NAMELIST = """
&nhyd_model
    config_time_integration_order = 3   ! third order
    config_dt = 7.2d2
    config_start_time = '2010-10-23_00:00:00'
    config_number_of_sub_steps = 2, config_dynamics_split_steps = 3
    config_h_mom_eddy_visc4 = 1.0e10
    config_horiz_mixing = '2d_fixed'
    config_monotonic = .false.
/
&damping
    config_zd = 22000.0
    config_xnutr = 0.2
/
"""


def test_namelist_parsing(tmp_path):
    p = tmp_path / "namelist.atmosphere"
    p.write_text(NAMELIST)
    cfg = gb.load_config_from_namelist(p)
    assert cfg["config_time_integration_order"] == 3 and cfg["config_dt"] == 720.0
    assert cfg["config_number_of_sub_steps"] == 2 and cfg["config_dynamics_split_steps"] == 3
    assert cfg["config_h_mom_eddy_visc4"] == 1.0e10 and cfg["config_horiz_mixing"] == "2d_fixed"
    assert cfg["config_monotonic"] is False and cfg["config_start_time"] == "2010-10-23_00:00:00"
    assert cfg["config_zd"] == 22000.0


def test_namelist_rejections(tmp_path):
    p = tmp_path / "nl"
    p.write_text("&nhyd_model\n config_dt = 600.0\n stray_key = 1\n/\n")
    with pytest.raises(gb.MpasStrictModeError):
        gb.load_config_from_namelist(p)
    with pytest.warns(UserWarning):
        assert gb.load_config_from_namelist(p, strict=False)["config_dt"] == 600.0
    p.write_text("&physics\n config_physics_suite = 'mesoscale_reference'\n/\n")
    with pytest.raises(gb.MpasUnsupportedCapabilityError):
        gb.load_config_from_namelist(p)
    with pytest.raises(FileNotFoundError):
        gb.load_config_from_namelist(tmp_path / "missing")


def test_load_initial_state_matches_reference_loader():
    from mpas_dycore_pytorch_gb300.cases import CaseSpec, make_case
    meta, st, _ = load_case("g2_mono")
    ref = group(st, "loaded")
    init, grid = make_case(CaseSpec(**meta["spec"]))
    state, mesh = gb.load_initial_state(init, grid, config=meta["config"])
    merged = dict(mesh)
    merged.update(state)
    for k in ("u", "theta", "scalars", "adv_coefs", "advCellsForEdge", "coeffs_reconstruct", "zb_cell", "rho_base"):
        g = merged[k].numpy() if isinstance(merged[k], torch.Tensor) else np.asarray(merged[k])
        assert g.shape == ref[k].shape, k
        assert np.abs(g - ref[k]).max() <= 1e-14 * max(np.abs(ref[k]).max(), 1e-300), k
    with pytest.raises(gb.MpasMissingFieldError):
        gb.load_initial_state({"u": np.zeros(3)}, grid, config=meta["config"])
    with pytest.raises(FileNotFoundError):
        gb.load_initial_state("no-such-init.nc", "no-such-grid.nc")


@pytest.mark.parametrize("name", ["read_history", "read_restart"])
def test_netcdf_readers_report_missing_files(name, tmp_path):
    with pytest.raises(FileNotFoundError):
        getattr(gb, name)(tmp_path / "x.nc")
