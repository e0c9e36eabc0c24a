"""Autotuned tile shapes: the u tendency agrees across levels-per-thread tiles to the
rounding of one fused multiply-add (the compiler fuses differently in the tiled kernel),
the step stays within the parity bound, and the autotuner picks one of the candidates
and reports their times."""

import ctypes as C

import numpy as np
import pytest
import torch

from gpu_helpers import need_gpu

pytestmark = pytest.mark.gpu

# tend_u after one dyn_tend call: relative max difference between tiles
TILE_TOL = {"float64": 1e-15, "mixed": 1e-6}
# all state fields after 2 steps: relative L2 (float64: the parity bound; mixed: its bound)
STEP_TOL = {"float64": 1e-12, "mixed": 1e-5}


def _model(precision, tile):
    from mpas_dycore_pytorch_gb300.api import Model
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.loader import load_case
    cfg = {"config_time_integration_order": 3, "config_len_disp": 120000.0, "config_monotonic": True,
           "config_dt": 600.0}
    st, _ = load_case(CaseSpec(level=4, nlev=23, seed=4, n_bumps=3, n_tracers=2), cfg, as_torch=False)
    m = Model(st, cfg, 600.0, num_scalars=2, precision=precision)
    m.prepare(st)
    m.cstruct.tile_tend_u = tile
    return m


@pytest.mark.parametrize("precision", ("float64", "mixed"))
def test_tiles_agree(precision):
    need_gpu()
    from mpas_dycore_pytorch_gb300.device import STATE_KEYS
    tend, state = {}, {}
    for tile in (1, 2, 4):
        m = _model(precision, tile)
        m.call("mpasg_dyn_tend", C.c_int(2))
        torch.cuda.synchronize()
        tend[tile] = m.state.f["tend_u"].clone()
        for _ in range(2):
            m.step()
        state[tile] = {k: m.state.f[k][:-1].double().cpu().numpy() for k in STATE_KEYS}
    scale = tend[1].abs().max().item()
    for tile in (2, 4):
        assert (tend[tile] - tend[1]).abs().max().item() <= TILE_TOL[precision] * scale, tile
        for k in STATE_KEYS:
            ref = state[1][k]
            den = max(np.linalg.norm(ref), 1e-300)
            assert np.linalg.norm(state[tile][k] - ref) / den <= STEP_TOL[precision], (tile, k)


def test_autotune_picks_a_candidate():
    need_gpu()
    m = _model("float64", 1)
    res = m.autotune()
    assert res["tend_u_levels_per_thread"] in (1, 2, 4)
    assert all(t > 0 for t in res["tend_u_ms"].values())
