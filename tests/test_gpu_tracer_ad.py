"""Derivatives of run_simulation with respect to the transported scalars on the GPU.

Against the reference's own ``run_simulation.vjp`` / ``.jvp`` (golden
``tests/golden/scalars_ad_g2.npz``, made by ``make_golden_diag.py``: two steps of
g2_explicit, objective sum(weights * final scalars)), the JVP/VJP dot-product identity
on a level-3 mesh, and a central finite difference of the objective.
"""

import pathlib

import numpy as np
import pytest
import torch

from fixtures import group, load_case, rel_l2
from gpu_helpers import need_gpu

pytestmark = pytest.mark.gpu

GOLDEN = np.load(pathlib.Path(__file__).resolve().parent / "golden" / "scalars_ad_g2.npz")
GRAD_TOL = 1e-10  # float64 gradients against the reference VJP


def _case():
    meta, st, _ = load_case("g2_explicit")
    loaded = group(st, "loaded")
    state = {k: torch.as_tensor(v) for k, v in loaded.items()}
    state.update({k: v for k, v in meta["loaded_scalars"].items()})
    return state, meta


def test_vjp_matches_reference():
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import run_simulation
    state, meta = _case()
    w = torch.as_tensor(GOLDEN["weights"]).cuda()
    grads = run_simulation.vjp(state, state, lambda o: (o["scalars"] * w).sum(), track_keys=("scalars",),
                               config=meta["config"], dt=meta["dt"], nsteps=2)
    assert set(grads) == {"scalars"}
    got = grads["scalars"].cpu().numpy()
    assert got.shape == GOLDEN["vjp_scalars"].shape
    assert rel_l2(got, GOLDEN["vjp_scalars"]) <= GRAD_TOL


def test_jvp_matches_reference():
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import run_simulation
    state, meta = _case()
    tan = torch.as_tensor(GOLDEN["tangent"])
    out = run_simulation.jvp(state, state, {"scalars": tan}, config=meta["config"], dt=meta["dt"], nsteps=2)
    assert "scalars" in GOLDEN["jvp_keys"]
    assert rel_l2(out["scalars"].cpu().numpy(), GOLDEN["jvp_scalars"]) <= GRAD_TOL


def _level3(n_tracers=2):
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.loader import load_case as load
    cfg = {"config_time_integration_order": 3, "config_len_disp": 240000.0, "config_monotonic": False,
           "config_dt": 1200.0}
    st, _ = load(CaseSpec(level=3, nlev=16, seed=4, n_bumps=4, n_tracers=n_tracers, dz_bottom=200.0), cfg,
                 as_torch=False)
    return {k: (torch.as_tensor(v) if isinstance(v, np.ndarray) else v) for k, v in st.items()}, cfg


def test_dot_product_identity():
    """<J v, w> = <v, J^T w> through three steps (two scalars)."""
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import run_simulation
    st, cfg = _level3()
    g = torch.Generator().manual_seed(7)
    v = torch.randn(st["scalars"].shape, generator=g, dtype=torch.float64)
    w = torch.randn(st["scalars"].shape, generator=g, dtype=torch.float64).cuda()
    jv = run_simulation.jvp(st, st, {"scalars": v}, config=cfg, nsteps=3)["scalars"].cuda()
    jtw = run_simulation.vjp(st, st, lambda o: (o["scalars"] * w).sum(), track_keys=("scalars",), config=cfg,
                             nsteps=3)["scalars"].cuda()
    lhs = float((jv * w).sum())
    rhs = float((v.cuda() * jtw).sum())
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs))
    # the control: a perturbed transpose must fail the identity
    assert abs(float((v.cuda() * (jtw * 1.001)).sum()) - lhs) > 1e-6 * abs(lhs)


def test_central_difference_matches_vjp():
    """The objective is linear in the start scalars: central differences over h = 2^-20 ..
    2^-36 reproduce <grad, v> to rounding."""
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import run_simulation
    st, cfg = _level3(n_tracers=1)
    g = torch.Generator().manual_seed(11)
    v = torch.randn(st["scalars"].shape, generator=g, dtype=torch.float64)
    w = torch.rand(st["scalars"].shape, generator=g, dtype=torch.float64).cuda()
    grad = run_simulation.vjp(st, st, lambda o: (o["scalars"] * w).sum(), track_keys=("scalars",), config=cfg,
                              nsteps=2)["scalars"].cuda()
    dd = float((grad * v.cuda()).sum())

    def objective(x):
        s = dict(st)
        s["scalars"] = x
        out = run_simulation(s, s, cfg, nsteps=2, use_cuda_graph=False)
        return float((out["scalars"] * w).sum())

    errs = []
    for p in (20, 28, 36):
        h = 2.0 ** -p
        fd = (objective(st["scalars"] + h * v) - objective(st["scalars"] - h * v)) / (2 * h)
        errs.append(abs(fd - dd) / abs(dd))
    assert min(errs) <= 1e-6, errs


def test_mixed_precision_derivatives_within_stated_error():
    """The mixed form's scalar VJP / JVP (float32 stencils in the taped forward and the
    tangent replay, float64 transposed transport) against the reference's float64 VJP /
    JVP: the stated bound for mixed-precision gradients is 1e-4."""
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import run_simulation
    state, meta = _case()
    cfg = dict(meta["config"], config_precision="mixed")
    w = torch.as_tensor(GOLDEN["weights"]).cuda()
    g = run_simulation.vjp(state, state, lambda o: (o["scalars"] * w).sum(), track_keys=("scalars",), config=cfg,
                           dt=meta["dt"], nsteps=2)["scalars"].cpu().numpy()
    t = run_simulation.jvp(state, state, {"scalars": torch.as_tensor(GOLDEN["tangent"])}, config=cfg, dt=meta["dt"],
                           nsteps=2)["scalars"].cpu().numpy()
    eg, et = rel_l2(g, GOLDEN["vjp_scalars"]), rel_l2(t, GOLDEN["jvp_scalars"])
    assert eg <= 1e-4 and et <= 1e-4, (eg, et)
    assert max(eg, et) > 1e-12  # float32 arithmetic really ran


def test_autograd_through_a_differentiable_run():
    """run_simulation(differentiable=True) with the start scalars requiring grad: the
    end scalars equal the plain run's, and backward() gives the reference's VJP (the same
    numbers as run_simulation.vjp)."""
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import run_simulation
    state, meta = _case()
    w = torch.as_tensor(GOLDEN["weights"]).cuda()
    x = state["scalars"].clone().requires_grad_(True)
    st = dict(state)
    st["scalars"] = x
    out = run_simulation(st, state, meta["config"], meta["dt"], nsteps=2, differentiable=True)
    assert out["scalars"].requires_grad
    plain = run_simulation(state, state, meta["config"], meta["dt"], nsteps=2)
    assert torch.equal(out["scalars"].detach(), plain["scalars"])
    (out["scalars"] * w).sum().backward()
    assert rel_l2(x.grad.numpy(), GOLDEN["vjp_scalars"]) <= GRAD_TOL
    via_vjp = run_simulation.vjp(state, state, lambda o: (o["scalars"] * w).sum(), track_keys=("scalars",),
                                 config=meta["config"], dt=meta["dt"], nsteps=2)["scalars"]
    assert torch.equal(x.grad, via_vjp.to(x.grad.device))


GOLDEN_C = np.load(pathlib.Path(__file__).resolve().parent / "golden" / "scalars_ad_g2_coupled.npz")


def _coupled_case():
    meta, st, _ = load_case("g2_coupled")
    state = {k: torch.as_tensor(v) for k, v in group(st, "loaded").items()}
    state.update(meta["loaded_scalars"])
    return state, dict(meta["config"], config_monotonic=False), float(meta["dt"])


def test_coupled_mode_vjp_and_jvp_match_reference():
    """Coupled transport (the scalars advance inside every RK stage with that stage's
    fluxes): the stage-by-stage adjoint and the replayed tangent against the reference's
    run_simulation.vjp / .jvp (golden scalars_ad_g2_coupled.npz, two steps)."""
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import run_simulation
    state, cfg, dt = _coupled_case()
    w = torch.as_tensor(GOLDEN_C["weights"]).cuda()
    g = run_simulation.vjp(state, state, lambda o: (o["scalars"] * w).sum(), track_keys=("scalars",), config=cfg,
                           dt=dt, nsteps=2)["scalars"].cpu().numpy()
    assert rel_l2(g, GOLDEN_C["vjp_scalars"]) <= GRAD_TOL
    t = run_simulation.jvp(state, state, {"scalars": torch.as_tensor(GOLDEN_C["tangent"])}, config=cfg, dt=dt,
                           nsteps=2)["scalars"].cpu().numpy()
    assert rel_l2(t, GOLDEN_C["jvp_scalars"]) <= GRAD_TOL


def test_coupled_mode_dot_product_identity():
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import run_simulation
    st, cfg = _level3()
    cfg = dict(cfg, config_split_dynamics_transport=False)
    g = torch.Generator().manual_seed(17)
    v = torch.randn(st["scalars"].shape, generator=g, dtype=torch.float64)
    w = torch.randn(st["scalars"].shape, generator=g, dtype=torch.float64).cuda()
    jv = run_simulation.jvp(st, st, {"scalars": v}, config=cfg, nsteps=3)["scalars"].cuda()
    jtw = run_simulation.vjp(st, st, lambda o: (o["scalars"] * w).sum(), track_keys=("scalars",), config=cfg,
                             nsteps=3)["scalars"].cuda()
    lhs = float((jv * w).sum())
    rhs = float((v.cuda() * jtw).sum())
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs))
