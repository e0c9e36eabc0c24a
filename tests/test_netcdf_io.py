"""History and restart files (``netcdf_io.py``): round trips of a complete step boundary
(the golden g2_explicit state after two steps), the checks the reference's readers and
writers make (restart.py, output_writer.py), and the integrity digests."""

import numpy as np
import pytest
import torch

from fixtures import group, load_case

import mpas_dycore_pytorch_gb300 as gb
from mpas_dycore_pytorch_gb300 import netcdf_io as io
from mpas_dycore_pytorch_gb300.api import resolved_config
from mpas_dycore_pytorch_gb300.boundary import MARKER, has_complete_step_boundary, mark_complete_step_boundary


def _torchify(d):
    out = {}
    for k, v in d.items():
        if isinstance(v, np.ndarray):
            out[k] = torch.as_tensor(v) if v.ndim > 0 else v.item()
        else:
            out[k] = v
    return out


@pytest.fixture(scope="module")
def case():
    meta, st, _ = load_case("g2_explicit")
    mesh = _torchify(group(st, "loaded"))
    state = _torchify(group(st, "prepared"))
    state.update(_torchify(group(st, "step2")))
    # bound as run_timestep binds the boundary it returns
    mark_complete_step_boundary(state, mesh=mesh, config=resolved_config(meta["config"]), dt=float(meta["dt"]))
    return state, mesh, meta["config"], float(meta["dt"])


def _write(tmp_path, case, name="r.nc", **kw):
    state, mesh, cfg, dt = case
    path = tmp_path / name
    args = dict(config=cfg, dt=dt, model_time_seconds=2 * dt)
    args.update(kw)
    gb.write_restart(state, mesh, path, "2000-01-01_01:00:00", **args)
    return path


def test_restart_round_trip_is_exact(tmp_path, case):
    state, mesh, cfg, dt = case
    path = _write(tmp_path, case)
    back, xtime = gb.read_restart(path, mesh=mesh, config=cfg, dt=dt)
    assert xtime == "2000-01-01_01:00:00"
    assert back["initial_time"] == "2000-01-01_00:00:00"
    assert back["_restart_model_time_seconds"] == 2 * dt
    nc = int(mesh["nCells"])
    for k, v in state.items():
        if not isinstance(v, torch.Tensor):
            continue
        got = back[k]
        assert got.dtype == v.dtype and got.shape == v.shape, k
        rowed = k in io.FIELD_DIMS and any(d in ("nCells", "nEdges", "nVertices") for d in io.FIELD_DIMS[k][:2])
        if rowed:
            assert torch.equal(got[:-1], v[:-1]), k  # active rows; the padding row is rebuilt
        else:
            assert torch.equal(got, v), k
    assert torch.all(back["rho_zz"][nc] == 1.0)
    assert torch.all(back["u"][-1] == 0.0)
    # a complete boundary, bound to the file's identity
    assert has_complete_step_boundary(back, mesh=mesh, config=resolved_config(cfg), dt=dt)


def test_restart_file_is_netcdf3_with_the_reference_schema(tmp_path, case):
    from scipy.io import netcdf_file
    path = _write(tmp_path, case)
    assert path.read_bytes()[:4] == b"CDF\x02"
    f = netcdf_file(str(path), "r", mmap=False)
    try:
        assert f.restart_schema == b"MPAS-PyTorch restart schema v1"
        assert int(f.restart_schema_version) == 1
        assert int(f.complete_step_boundary) == 1
        assert f.variables["u"].dimensions == ("Time", "nEdges", "nVertLevels")
        assert f.variables["w"].dimensions == ("Time", "nCells", "nVertLevelsP1")
        assert f.variables["scalars"].dimensions == ("Time", "nCells", "nVertLevels", "nScalars")
        assert f.variables["xtime"].dimensions == ("Time", "StrLen")
        assert f.variables["u"].data.shape[1] == int(case[1]["nEdges"])  # active rows only
        assert len(f._attributes["restart_payload_sha256"]) == 64
    finally:
        f.close()


def test_restart_refuses_overwrite_and_clobbers_on_request(tmp_path, case):
    path = _write(tmp_path, case)
    with pytest.raises(FileExistsError):
        _write(tmp_path, case)
    _write(tmp_path, case, clobber=True)
    assert not list(tmp_path.glob(".*.tmp"))


def test_restart_missing_fields_and_mid_step_state_are_rejected(tmp_path, case):
    state, mesh, cfg, dt = case
    bad = {k: v for k, v in state.items() if k != "rtheta_base"}
    mesh2 = {k: v for k, v in mesh.items() if k != "rtheta_base"}
    with pytest.raises(gb.MpasMissingFieldError) as ei:
        gb.write_restart(bad, mesh2, tmp_path / "a.nc", "2000-01-01_01:00:00", config=cfg, dt=dt)
    assert "rtheta_base" in ei.value.fields
    # a non-zero acoustic carry without the boundary snapshot is a mid-RK3 savepoint
    mid = {k: v for k, v in state.items() if k not in ("v", "ruAvg")}
    mid["rho_pp"] = torch.ones_like(state["rho_zz"])
    with pytest.raises(gb.MpasConfigError, match="mid-RK3"):
        gb.write_restart(mid, mesh, tmp_path / "b.nc", "2000-01-01_01:00:00", config=cfg, dt=dt)
    with pytest.raises(gb.MpasConfigError):
        gb.write_restart(state, mesh, tmp_path / "c.nc", "not a time", config=cfg, dt=dt)
    with pytest.raises(gb.MpasConfigError):
        gb.write_restart(state, mesh, tmp_path / "d.nc", "2000-01-01_01:00:00", config=cfg, dt=-1.0)
    nonfinite = dict(state)
    nonfinite["theta_m"] = state["theta_m"].clone()
    nonfinite["theta_m"][0, 0] = float("nan")
    with pytest.raises(gb.MpasConfigError):
        gb.write_restart(nonfinite, mesh, tmp_path / "e.nc", "2000-01-01_01:00:00", config=cfg, dt=dt)
    assert not (tmp_path / "e.nc").exists()


def test_restart_reader_checks_identity_and_integrity(tmp_path, case):
    state, mesh, cfg, dt = case
    path = _write(tmp_path, case)
    with pytest.raises(gb.MpasConfigError, match="configuration digest"):
        gb.read_restart(path, config=dict(cfg, config_dt=dt + 1.0))
    with pytest.raises(gb.MpasConfigError, match="timestep"):
        gb.read_restart(path, dt=dt / 2)
    other = dict(mesh)
    other["dcEdge"] = mesh["dcEdge"] * 1.0000001
    with pytest.raises(gb.MpasMeshMismatchError):
        gb.read_restart(path, mesh=other)
    with pytest.raises(gb.MpasMeshMismatchError):
        gb.read_restart(path, mesh=dict(mesh, nVertLevels=int(mesh["nVertLevels"]) + 1))
    with pytest.raises(gb.MpasDeviceError):
        gb.read_restart(path, device="meta")
    # one flipped byte in the payload breaks the integrity digest
    raw = bytearray(path.read_bytes())
    raw[len(raw) // 2] ^= 0x01  # inside the float64 payload
    bad = tmp_path / "tampered.nc"
    bad.write_bytes(bytes(raw))
    with pytest.raises(gb.MpasConfigError, match="digest"):
        gb.read_restart(bad)
    with pytest.raises(FileNotFoundError):
        gb.read_restart(tmp_path / "missing.nc")


def test_netcdf4_files_need_netcdf4(tmp_path):
    p = tmp_path / "hdf5.nc"
    p.write_bytes(b"\x89HDF\r\n\x1a\n" + bytes(64))
    with pytest.raises(gb.MpasUnsupportedCapabilityError):
        gb.read_restart(p)
    with pytest.raises(gb.MpasUnsupportedCapabilityError):
        gb.read_history(p)


def test_history_fields_metadata_and_time(tmp_path, case):
    state, mesh, cfg, dt = case
    path = tmp_path / "h.nc"
    gb.write_history(path, state, mesh, xtime="2000-01-01_01:00:00", config=cfg, dt=dt, model_time_seconds=3600.0,
                     global_attrs={"title": "g2"})
    h = gb.read_history(path)
    f, d, a = h["fields"], h["dimensions"], h["attributes"]
    nc, ne, L = int(mesh["nCells"]), int(mesh["nEdges"]), int(mesh["nVertLevels"])
    assert d["Time"] is None and d["nCells"] == nc and d["nVertLevelsP1"] == L + 1
    assert a["history_schema"] == io.HISTORY_SCHEMA and a["title"] == "g2"
    np.testing.assert_array_equal(f["u"][0], state["u"].numpy()[:ne, :L])
    qv = state["scalars"].numpy()[:nc, :L, 0]
    np.testing.assert_array_equal(f["theta"][0], state["theta_m"].numpy()[:nc, :L] / (1.0 + io.RVORD * qv))
    np.testing.assert_array_equal(f["rho"][0], state["rho_zz"].numpy()[:nc, :L] * mesh["zz"].numpy()[:nc, :L])
    np.testing.assert_array_equal(f["pressure"][0], state["pressure_p"].numpy()[:nc, :L] +
                                  state["pressure_base"].numpy()[:nc, :L])
    assert float(f["time"][0]) == 3600.0
    sel = tmp_path / "sel.nc"
    gb.write_history(sel, state, mesh, xtime="2000-01-01_01:00:00", fields=["u", "scalars"], dt=dt)
    assert set(gb.read_history(sel)["fields"]) == {"u", "qv", "time", "xtime"}


def test_history_rejections(tmp_path, case):
    state, mesh, cfg, dt = case
    with pytest.raises(gb.MpasConfigError, match="Unsupported history fields"):
        gb.write_history(tmp_path / "a.nc", state, mesh, fields=["nonsense"])
    with pytest.raises(gb.MpasConfigError, match="Reserved"):
        gb.write_history(tmp_path / "b.nc", state, mesh, global_attrs={"package_version": "x"})
    with pytest.raises(gb.MpasMissingFieldError):
        gb.write_history(tmp_path / "c.nc", {k: v for k, v in state.items() if k != "theta_m"},
                         {k: v for k, v in mesh.items() if k != "theta_m"}, fields=["theta"])
    gb.write_history(tmp_path / "d.nc", state, mesh, xtime="2000-01-01_01:00:00", dt=dt)
    with pytest.raises(FileExistsError):
        gb.write_history(tmp_path / "d.nc", state, mesh, xtime="2000-01-01_01:00:00", dt=dt)


def test_case_files_load_like_the_in_memory_case(tmp_path):
    """The synthetic case written as MPAS grid / initial-condition files (NetCDF-3) loads
    to the same state and mesh as the in-memory fields."""
    from mpas_dycore_pytorch_gb300.cases import CaseSpec, make_case, write_case_files
    spec = CaseSpec(level=2, nlev=12, seed=3, n_bumps=4, n_tracers=2)
    init_path, grid_path = write_case_files(spec, tmp_path)
    assert init_path.read_bytes()[:3] == b"CDF" and grid_path.read_bytes()[:3] == b"CDF"
    init, grid = make_case(spec)
    cfg = {"config_dt": 1800.0}
    s1, m1 = gb.load_initial_state(init, grid, config=cfg)
    s2, m2 = gb.load_initial_state(str(init_path), str(grid_path), config=cfg)
    for d1, d2 in ((s1, s2), (m1, m2)):
        for k, a in d1.items():
            b = d2[k]
            if isinstance(a, torch.Tensor):
                assert a.dtype == b.dtype and a.shape == b.shape and torch.equal(a, b), k
            else:
                assert a == b, k
    fields = io.read_mpas_fields(init_path)
    assert fields["nCells"] == grid["nCells"] and fields["u"].shape == init["u"].shape
    with pytest.raises(FileExistsError):
        write_case_files(spec, tmp_path)
