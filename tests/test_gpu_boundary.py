"""Continuation from a returned step boundary on the GPU (reference state.py:194-264,
atmosphere_model.py:829-898), against the reference's own continuations of the
g2_explicit case (``tests/golden/make_golden_boundary.py``):

* the device digest of a tensor equals the host digest of the same bytes;
* one step and one more from the returned (bound) boundary equal two steps, bit for bit;
* a boundary whose prognostics theta_m and u were edited is re-derived before the step,
  and matches the reference's continuation of the same edit (relative L2 1e-12, the bound
  of the step parity tests);
* an edited diagnostic and another time step are rejected with the reference's messages;
* the restart writer refuses an edited boundary.
"""

import json

import numpy as np
import pytest
import torch

from fixtures import GOLDEN, group, load_case, step_tol
from gpu_helpers import need_gpu

pytestmark = pytest.mark.gpu

CASE = "g2_explicit"


def _setup():
    meta, st, _ = load_case(CASE)
    state = {k: torch.as_tensor(v) for k, v in group(st, "loaded").items()}
    state.update(meta["loaded_scalars"])
    return state, meta["config"], float(meta["dt"])


def _rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_device_digest_equals_host_digest():
    need_gpu()
    from mpas_dycore_pytorch_gb300 import boundary as bd
    rng = np.random.default_rng(3)
    for n in (0, 1, 7, 8, 9, 4096, 1000003, 3 * (1 << 20) + 5):
        raw = rng.integers(0, 256, n, dtype=np.uint8)
        host = bd._snapshot({"x": raw})["x"][2]
        dev = bd._snapshot({"x": torch.from_numpy(raw).cuda()})["x"][2]
        assert host == dev, n
    x = torch.randn(1000, 7, dtype=torch.float64, device="cuda")
    v = x[:, 2]  # a strided view is digested as its contiguous bytes
    assert bd._snapshot({"v": v})["v"][2] == bd._snapshot({"v": v.cpu().contiguous()})["v"][2]


def test_continuation_from_the_returned_boundary():
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import resolved_config, run_simulation
    from mpas_dycore_pytorch_gb300.boundary import has_complete_step_boundary
    from mpas_dycore_pytorch_gb300.device import STATE_KEYS
    state, cfg, dt = _setup()
    b1 = run_simulation(state, state, cfg, dt, nsteps=1)
    # bound to the mesh, the full (defaults filled in) configuration and the time step
    assert has_complete_step_boundary(b1, mesh=state, config=resolved_config(cfg), dt=dt)
    assert not has_complete_step_boundary(b1, dt=dt / 2)
    cont = run_simulation(b1, state, cfg, dt, nsteps=1)
    assert has_complete_step_boundary(b1)  # the input boundary is not changed
    straight = run_simulation(state, state, cfg, dt, nsteps=2)
    for k in STATE_KEYS:
        assert torch.equal(straight[k][:-1], cont[k][:-1]), k
    gold = dict(np.load(GOLDEN / f"boundary_{CASE}.npz"))
    for k in ("u", "theta_m", "rho_zz", "w", "pressure_p"):
        err = _rel(cont[k][:-1].cpu().numpy(), gold[f"cont/{k}"][:-1])
        print(f"continued {k}: rel L2 {err:.2e}")
        assert err <= step_tol(CASE, k), (k, err)


def test_edited_prognostics_are_rederived_as_the_reference_does():
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import run_simulation
    state, cfg, dt = _setup()
    meta = json.loads((GOLDEN / f"boundary_{CASE}.json").read_text())
    gold = dict(np.load(GOLDEN / f"boundary_{CASE}.npz"))
    b1 = run_simulation(state, state, cfg, dt, nsteps=1)
    as_is = run_simulation(b1, state, cfg, dt, nsteps=1)
    c, k, f = meta["edit_theta_m"]
    e, ku, du = meta["edit_u"]
    ed = dict(b1)
    ed["theta_m"] = b1["theta_m"].clone()
    ed["theta_m"][c, k] *= f
    ed["u"] = b1["u"].clone()
    ed["u"][e, ku] += du
    out = run_simulation(ed, state, cfg, dt, nsteps=1)
    worst = 0.0
    for key in ("u", "w", "theta_m", "rho_zz", "pressure_p", "exner", "rho_p", "rtheta_p", "ru", "rw", "v",
                "divergence", "vorticity", "ke", "pv_edge", "h_edge", "scalars"):
        err = _rel(out[key][:-1].cpu().numpy(), gold[f"edit/{key}"][:-1])
        print(f"edited continuation {key}: rel L2 {err:.2e}")
        assert err <= step_tol(CASE, key), (key, err)
        worst = max(worst, err)
    # the edit reached the step (not continued as the unedited boundary)
    assert _rel(out["theta_m"][:-1].cpu().numpy(), as_is["theta_m"][:-1].cpu().numpy()) > 1e-8
    # the control: the edited prognostics continued with the old diagnostics (no
    # re-derivation) miss the reference's continuation by far more than the bound
    from mpas_dycore_pytorch_gb300.api import _simulate
    stale = _simulate(ed, state, cfg, dt, 1, "cuda", None, False, None, None, False, bound=False)
    miss = max(_rel(stale[key][:-1].cpu().numpy(), gold[f"edit/{key}"][:-1]) for key in ("rho_p", "ru", "exner"))
    print(f"stale-diagnostics control: worst rel L2 {miss:.2e}")
    assert miss > 1e3 * max(worst, 1e-15)


def test_edited_diagnostic_and_other_time_step_are_rejected(tmp_path):
    need_gpu()
    import mpas_dycore_pytorch_gb300 as gb
    from mpas_dycore_pytorch_gb300.api import run_simulation
    from mpas_dycore_pytorch_gb300.errors import MpasConfigError
    state, cfg, dt = _setup()
    meta = json.loads((GOLDEN / f"boundary_{CASE}.json").read_text())
    b1 = run_simulation(state, state, cfg, dt, nsteps=1)
    ed = dict(b1)
    ed["exner"] = b1["exner"].clone()
    ed["exner"][5, 3] *= 1.0001
    msg = meta["messages"]["diagnostic_edit"].split(": ", 1)[1]
    with pytest.raises(MpasConfigError, match=msg):
        run_simulation(ed, state, cfg, dt, nsteps=1)
    msg = meta["messages"]["other_dt"].split(": ", 1)[1]
    with pytest.raises(MpasConfigError, match=msg):
        run_simulation(b1, state, cfg, dt / 2, nsteps=1)
    with pytest.raises(MpasConfigError, match=msg):
        run_simulation(b1, state, dict(cfg, config_len_disp=1.0), dt, nsteps=1)
    prog = dict(b1)
    prog["u"] = b1["u"] * 1.0001
    with pytest.raises(MpasConfigError, match="edited timestep boundary"):
        gb.write_restart(prog, state, tmp_path / "r.nc", "2000-01-01_01:00:00", config=cfg, dt=dt,
                         model_time_seconds=dt)
