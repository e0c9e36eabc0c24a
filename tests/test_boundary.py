"""Binding of a returned step boundary (``boundary.py``; reference state.py:66-264) on the
host: the value digest, and the marks and checks that ``run_simulation`` and the restart
writer make.  The device digest and the continuation on the GPU are in
``test_gpu_boundary.py``."""

import numpy as np
import pytest
import torch

from mpas_dycore_pytorch_gb300 import boundary as bd
from mpas_dycore_pytorch_gb300.errors import MpasConfigError


def _state(seed=0):
    g = torch.Generator().manual_seed(seed)
    return {"u": torch.randn(9, 4, dtype=torch.float64, generator=g),
            "w": torch.randn(5, 5, dtype=torch.float64, generator=g),
            "rho_zz": torch.rand(5, 4, dtype=torch.float64, generator=g) + 1.0,
            "theta_m": torch.rand(5, 4, dtype=torch.float64, generator=g) + 300.0,
            "scalars": torch.rand(5, 4, 2, dtype=torch.float64, generator=g),
            "exner": torch.rand(5, 4, dtype=torch.float64, generator=g),
            "cellsOnEdge": np.arange(18, dtype=np.int32).reshape(9, 2),
            "nCells": 4, "config_tag": "x"}


def test_digest_tracks_every_byte_and_nothing_else():
    raw = np.random.default_rng(1).integers(0, 256, 1003, dtype=np.uint8)
    base = bd._finish(*bd._lanes_host(raw), raw.size)
    assert base == bd._finish(*bd._lanes_host(raw.copy()), raw.size)
    for i in (0, 7, 8, 500, 1002):  # every word, including the zero-padded tail
        r2 = raw.copy()
        r2[i] ^= 1
        assert bd._finish(*bd._lanes_host(r2), r2.size) != base
    # swapping two words changes it (the index is mixed in), so does the length
    r3 = raw.copy()
    r3[:8], r3[8:16] = raw[8:16], raw[:8]
    assert bd._finish(*bd._lanes_host(r3), r3.size) != base
    assert bd._finish(*bd._lanes_host(raw[:1002]), 1002) != base
    # a trailing zero byte is not the same as no byte
    z = np.zeros(8, dtype=np.uint8)
    assert bd._finish(*bd._lanes_host(z[:7]), 7) != bd._finish(*bd._lanes_host(z), 8)


def test_marked_state_survives_a_clone_and_catches_edits():
    st = _state()
    bd.mark_complete_step_boundary(st, mesh={"x": np.arange(3.0)}, config={"a": 1}, dt=60.0)
    assert bd.has_complete_step_boundary(st)
    assert bd.has_complete_step_boundary(st, mesh={"x": np.arange(3.0)}, config={"a": 1}, dt=60.0)
    assert not bd.has_complete_step_boundary(st, dt=30.0)
    assert not bd.has_complete_step_boundary(st, config={"a": 2})
    clone = {k: (v.clone() if isinstance(v, torch.Tensor) else v) for k, v in st.items()}
    assert bd.has_complete_step_boundary(clone)
    # one ulp of one prognostic: no longer complete, but its support is unedited
    st["u"][3, 1] = torch.nextafter(st["u"][3, 1], torch.tensor(np.inf, dtype=torch.float64))
    assert not bd.has_complete_step_boundary(st)
    bd.require_unedited_boundary_support(st)
    # -0.0 for +0.0 is a byte edit
    st2 = _state()
    st2["exner"][0, 0] = 0.0
    bd.mark_complete_step_boundary(st2)
    st2["exner"][0, 0] = -0.0
    assert not bd.has_complete_step_boundary(st2)
    with pytest.raises(MpasConfigError, match="diagnostics or support inputs were edited"):
        bd.require_unedited_boundary_support(st2)


def test_support_scalars_and_arrays_are_bound():
    for edit in ("nCells", "config_tag", "cellsOnEdge"):
        st = _state()
        bd.mark_complete_step_boundary(st)
        if edit == "cellsOnEdge":
            st[edit] = st[edit].copy()
            st[edit][0, 0] = 5
        else:
            st[edit] = 5 if edit == "nCells" else "y"
        with pytest.raises(MpasConfigError, match="support inputs were edited"):
            bd.require_unedited_boundary_support(st)


def test_continuation_identity_and_binding_tag():
    st = _state()
    mesh = {"x": np.arange(3.0), "n": 3}
    bd.mark_complete_step_boundary(st, mesh=mesh, config={"a": 1, "_private": 2}, dt=60.0)
    bd.require_boundary_continuation_identity(st, mesh=mesh, config={"a": 1, "_other": 3}, dt=60.0)
    for kw in (dict(mesh={"x": np.arange(4.0), "n": 3}, config={"a": 1}, dt=60.0),
               dict(mesh=mesh, config={"a": 2}, dt=60.0), dict(mesh=mesh, config={"a": 1}, dt=61.0),
               dict(mesh=None, config={"a": 1}, dt=60.0)):
        with pytest.raises(MpasConfigError, match="continuation identity mismatch"):
            bd.require_boundary_continuation_identity(st, **kw)
    st[bd.MARKER] = dict(st[bd.MARKER], binding="legacy")
    assert not bd.has_complete_step_boundary(st)
    with pytest.raises(MpasConfigError, match="binding is unsupported"):
        bd.require_unedited_boundary_support(st)


def test_alias_may_follow_its_primary_only():
    st = _state()
    st["t"] = st["theta_m"].clone()
    bd.mark_complete_step_boundary(st)
    st["theta_m"] = st["theta_m"] + 1.0
    bd.require_unedited_boundary_support(st)  # the alias unchanged
    st["t"] = st["t"] + 2.0
    with pytest.raises(MpasConfigError, match="alias was edited"):
        bd.require_unedited_boundary_support(st)
    st["t"] = st["theta_m"].clone()  # follows the edited primary exactly
    bd.require_unedited_boundary_support(st)
    del st["t"]
    with pytest.raises(MpasConfigError, match="alias inventory changed"):
        bd.require_unedited_boundary_support(st)


def test_a_boundary_without_a_prognostic_cannot_be_marked():
    st = _state()
    del st["scalars"]
    with pytest.raises(MpasConfigError, match="lacks tensor 'scalars'"):
        bd.mark_complete_step_boundary(st)
