"""Restart continuation on the GPU: two steps, a restart file, two more steps equal four
steps run straight through, bit for bit (the reference's 2 + 2 restart check,
examples/validate_model.py:568-611), and a history file of the result."""

import numpy as np
import pytest
import torch

from fixtures import group, load_case
from gpu_helpers import need_gpu

pytestmark = pytest.mark.gpu


def test_two_plus_two_steps_through_a_restart_file_are_bitwise(tmp_path):
    need_gpu()
    import mpas_dycore_pytorch_gb300 as gb
    from mpas_dycore_pytorch_gb300.api import run_simulation
    from mpas_dycore_pytorch_gb300.device import STATE_KEYS
    meta, st, _ = load_case("g2_explicit")
    state = {k: torch.as_tensor(v) for k, v in group(st, "loaded").items()}
    state.update(meta["loaded_scalars"])
    cfg, dt = meta["config"], float(meta["dt"])
    straight = run_simulation(state, state, cfg, dt, nsteps=4)
    half = run_simulation(state, state, cfg, dt, nsteps=2)
    path = tmp_path / "restart.nc"
    gb.write_restart(half, state, path, "2000-01-01_01:00:00", config=cfg, dt=dt, model_time_seconds=2 * dt)
    back, xtime = gb.read_restart(path, mesh=state, config=cfg, dt=dt)
    assert xtime == "2000-01-01_01:00:00"
    cont = run_simulation(back, state, cfg, dt, nsteps=2)
    for k in STATE_KEYS:
        a, b = straight[k][:-1].cpu(), cont[k][:-1].cpu()
        assert torch.equal(a, b), (k, float((a - b).abs().max()))
    # and the history of the result holds the same prognostics
    hist = tmp_path / "history.nc"
    gb.write_history(hist, cont, state, xtime="2000-01-01_02:00:00", dt=dt, model_time_seconds=4 * dt)
    h = gb.read_history(hist)["fields"]
    ne, L = int(state["nEdges"]), int(state["nVertLevels"])
    np.testing.assert_array_equal(h["u"][0], straight["u"][:ne, :L].cpu().numpy())
