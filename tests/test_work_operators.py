"""The reference-named keyword operators (``work.py``): the routine table and the checks
that run before any device work."""

from types import SimpleNamespace

import numpy as np
import pytest

from mpas_dycore_pytorch_gb300 import work
from mpas_dycore_pytorch_gb300.errors import MpasConfigError
from mpas_dycore_pytorch_gb300.stages import STAGES


def test_every_stage_has_its_reference_routine():
    assert sorted(k for k, _ in work.ROUTINES.values()) == sorted(STAGES)
    for routine in work.ROUTINES:
        op = getattr(work, routine)
        assert op.__name__ == routine and routine in work.__all__
        assert work.ROUTINES[routine][1] in op.__doc__


def test_operator_without_a_resident_mesh_is_rejected():
    work._context.clear()
    with pytest.raises(MpasConfigError, match="use_mesh"):
        work.atm_divergence_damping_3d(dts=1.0)


def test_operator_checks_dimensions_connectivity_and_options():
    mesh = {"cellsOnEdge": np.array([[0, 1], [1, 2], [2, 0]], dtype=np.int32), "nCells": 3}
    fake = SimpleNamespace(dmesh=SimpleNamespace(nCells=3, nEdges=3, nVertices=2, nVertLevels=4),
                           cfg={"config_smdiv": 0.1, "config_epssm": 0.1, "config_mix_full": True})
    work._context.clear()
    work._context.update(model=fake, mesh=mesh)
    ok = dict(nCells=3, nEdges=3, nVertLevels=4, cellsOnEdge=mesh["cellsOnEdge"].copy(), config_smdiv=0.1,
              epssm=0.1, config_mix_full=1, config_unknown_option=7)
    assert work._checked_model("r", ok) is fake
    with pytest.raises(MpasConfigError, match="nCells=4"):
        work._checked_model("r", dict(ok, nCells=4))
    coe = mesh["cellsOnEdge"].copy()
    coe[0] = coe[0, ::-1]
    with pytest.raises(MpasConfigError, match="cellsOnEdge"):
        work._checked_model("r", dict(ok, cellsOnEdge=coe))
    with pytest.raises(MpasConfigError, match="config_smdiv"):
        work._checked_model("r", dict(ok, config_smdiv=0.2))
    with pytest.raises(MpasConfigError, match="epssm"):
        work._checked_model("r", dict(ok, epssm=0.2))
    with pytest.raises(MpasConfigError, match="config_mix_full"):
        work._checked_model("r", dict(ok, config_mix_full=0))
    work._context.clear()
