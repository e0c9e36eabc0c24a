"""The dynamics gradient of the differentiation workload against central differences.

Recipe: level-5 mesh (10242 cells x 41 levels), the analytic dry state with 8 seeded theta
bumps, a 0.1 m/s sinusoidal w and the wind rounded to 16 significant bits (so that the
perturbations below are exactly representable where the reference's recipe needs it,
examples/validate_model.py:216-252), 24 steps at dt 900 s (RK3, 3 x 2 substeps).  The
functional is the area-weighted squared anomaly of the surface pressure at the final time
against the initial surface pressure.  Its gradient with respect to the initial u and theta
(run_simulation.vjp) is checked along a seeded random direction against central differences
of run_simulation over h = 2^-12 ... 2^-36 (the stated 2^-20 ... 2^-36 and the larger steps
that show the truncation side of the curve): it must reach a relative error <= 1e-7,
and a control that drops the theta part of the gradient must miss it by far.  The same
directional derivative from the forward mode (run_simulation.jvp, the functional's
derivative applied to the final tangents) must meet the reverse mode's within 1e-12: the
JVP/VJP identity on this workload.  The mixed form's gradient (its float32-stencil
trajectory, linearised in float64) must be within 1e-4 of the float64 gradient.
"""

import math

import numpy as np
import pytest
import torch

from gpu_helpers import need_gpu

pytestmark = pytest.mark.gpu

SPEC = dict(level=5, nlev=41, seed=2, n_bumps=8, n_tracers=1, w_sine=0.1, round_wind_bits=16)
CFG = {"config_time_integration_order": 3, "config_len_disp": 120000.0, "config_number_of_sub_steps": 2,
       "config_dynamics_split_steps": 3, "config_monotonic": False, "config_dt": 900.0}
NSTEPS = 24
H = [2.0 ** -e for e in range(12, 37, 2)]


def _setup():
    from mpas_dycore_pytorch_gb300.api import run_simulation
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.diagnostics import physics_interface_surface_pressure, surface_pressure_functional
    from mpas_dycore_pytorch_gb300.loader import load_case
    st, mesh = load_case(CaseSpec(**SPEC), CFG, as_torch=True)
    nc = int(st["nCells"])
    dev = torch.device("cuda")
    zz = st["zz"].to(dev, torch.float64)
    zgrid = st["zgrid"].to(dev, torch.float64)
    area = st["areaCell"].to(dev, torch.float64)

    def sp_of(out):
        rz = out["rho_zz"]
        return physics_interface_surface_pressure(nCells=nc, rho_zz=rz, zz=zz, qv=torch.zeros_like(rz),
                                                  pressure_p=out["pressure_p"], pressure_base=out["pressure_base"],
                                                  zgrid=zgrid)

    prepared = run_simulation(st, mesh, CFG, 900.0, nsteps=1, on_initial=lambda s: None)  # warm the path
    del prepared
    box = {}
    run_simulation(st, mesh, CFG, 900.0, nsteps=1,
                   on_initial=lambda s: box.update({k: v.clone() for k, v in s.items()
                                                    if isinstance(v, torch.Tensor) and v.is_cuda}))
    sp_ref = sp_of(box).detach()

    def objective(out):
        return surface_pressure_functional(sp_of(out), sp_ref, area, nc)

    return st, mesh, objective


def test_gradient_matches_central_differences():
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import run_simulation
    st, mesh, objective = _setup()
    grads = run_simulation.vjp(st, mesh, objective, track_keys=("u", "theta"), config=CFG, dt=900.0,
                               nsteps=NSTEPS)
    rng = np.random.default_rng(2)
    d = {}
    for k, scale in (("u", 1.0), ("theta", 0.1)):
        x = rng.standard_normal(tuple(st[k].shape)) * scale
        x[-1] = 0.0  # the padding row is not perturbed
        d[k] = torch.as_tensor(x)
    dJ = sum(float((grads[k].cpu() * d[k]).sum()) for k in d)
    # forward mode: the final tangents along d, contracted with the functional's derivative
    tan = run_simulation.jvp(st, mesh, {"u": d["u"], "theta": d["theta"]}, config=CFG, dt=900.0, nsteps=NSTEPS)
    final = run_simulation(st, mesh, CFG, 900.0, nsteps=NSTEPS)
    leaves = {k: final[k].detach().clone().requires_grad_(True) for k in ("rho_zz", "pressure_p")}
    gj = torch.autograd.grad(objective({**final, **leaves}), [leaves["rho_zz"], leaves["pressure_p"]])
    dJ_fwd = sum(float((g * tan[k].to(g.device)).sum()) for g, k in zip(gj, ("rho_zz", "pressure_p")))
    ident = abs(dJ_fwd - dJ) / abs(dJ)
    print(f"JVP/VJP identity: forward {dJ_fwd:.15e} reverse {dJ:.15e} rel {ident:.2e}")
    assert ident <= 1e-12, (dJ_fwd, dJ, ident)
    # sqrt(24) = 5-step checkpoint segments with one substep taped at a time: bit for bit
    nested = run_simulation.vjp(st, mesh, objective, track_keys=("u", "theta"),
                                config=dict(CFG, gradient_checkpointing=True), dt=900.0, nsteps=NSTEPS)
    for k in ("u", "theta"):
        assert torch.equal(nested[k], grads[k]), k
    # the mixed form's gradient against the float64 one
    mixed = run_simulation.vjp(st, mesh, objective, track_keys=("u", "theta"),
                               config=dict(CFG, config_precision="mixed"), dt=900.0, nsteps=NSTEPS)
    for k in ("u", "theta"):
        a, b = mixed[k][:-1].cpu().numpy(), grads[k][:-1].cpu().numpy()
        err = float(np.linalg.norm(a - b) / np.linalg.norm(b))
        print(f"mixed-form gradient {k}: rel L2 vs float64 {err:.3e}")
        assert err <= 1e-4, (k, err)
    rows = []
    for h in H:
        Js = []
        for sgn in (1.0, -1.0):
            s2 = dict(st)
            for k in d:
                s2[k] = st[k] + sgn * h * d[k]
            Js.append(float(objective(run_simulation(s2, mesh, CFG, 900.0, nsteps=NSTEPS))))
        fd = (Js[0] - Js[1]) / (2.0 * h)
        rows.append((h, fd, abs(fd - dJ) / abs(dJ)))
    for h, fd, err in rows:
        print(f"FD h=2^{int(round(math.log2(h)))} fd={fd:.12e} adjoint={dJ:.12e} rel_err={err:.3e}")
    errs = [r[2] for r in rows]
    assert min(errs) <= 1e-7, errs
    # failing control: without its theta part the directional derivative misses every point
    dJ_u = float((grads["u"].cpu() * d["u"]).sum())
    assert min(abs(fd - dJ_u) / abs(dJ) for _, fd, _ in rows) > 1e-3


def test_terrain_gradient_matches_central_differences():
    """Over terrain-following levels (a 1500 m cosine hill on the level-4 mesh, 26 levels,
    fixed-coefficient mixing, 4 steps at dt 1200 s): the gradient with respect to u and
    theta along a seeded direction against central differences over h = 2^-12 ... 2^-30,
    best point within 1e-7; the control without the theta part misses by far."""
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import run_simulation
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.diagnostics import physics_interface_surface_pressure, surface_pressure_functional
    from mpas_dycore_pytorch_gb300.loader import load_case
    spec = dict(level=4, nlev=26, dz_bottom=300.0, seed=6, n_bumps=8, n_tracers=1, w_sine=0.1,
                round_wind_bits=16, terrain=1500.0)
    cfg = {"config_time_integration_order": 3, "config_len_disp": 240000.0, "config_number_of_sub_steps": 2,
           "config_dynamics_split_steps": 3, "config_monotonic": False, "config_dt": 1200.0,
           "config_horiz_mixing": "2d_fixed", "config_h_mom_eddy_visc4": 1.0e11,
           "config_h_theta_eddy_visc4": 5.0e10, "config_h_theta_eddy_visc2": 4.0e4}
    nsteps = 4
    st, mesh = load_case(CaseSpec(**spec), cfg, as_torch=True)
    nc = int(st["nCells"])
    dev = torch.device("cuda")
    zz, zgrid, area = (st[k].to(dev, torch.float64) for k in ("zz", "zgrid", "areaCell"))

    def sp_of(out):
        rz = out["rho_zz"]
        return physics_interface_surface_pressure(nCells=nc, rho_zz=rz, zz=zz, qv=torch.zeros_like(rz),
                                                  pressure_p=out["pressure_p"], pressure_base=out["pressure_base"],
                                                  zgrid=zgrid)

    box = {}
    run_simulation(st, mesh, cfg, 1200.0, nsteps=1,
                   on_initial=lambda s: box.update({k: v.clone() for k, v in s.items()
                                                    if isinstance(v, torch.Tensor) and v.is_cuda}))
    sp_ref = sp_of(box).detach()

    def objective(out):
        return surface_pressure_functional(sp_of(out), sp_ref, area, nc)

    grads = run_simulation.vjp(st, mesh, objective, track_keys=("u", "theta"), config=cfg, dt=1200.0,
                               nsteps=nsteps)
    rng = np.random.default_rng(6)
    d = {}
    for k, scale in (("u", 1.0), ("theta", 0.1)):
        x = rng.standard_normal(tuple(st[k].shape)) * scale
        x[-1] = 0.0
        d[k] = torch.as_tensor(x)
    dJ = sum(float((grads[k].cpu() * d[k]).sum()) for k in d)
    rows = []
    for h in [2.0 ** -e for e in range(12, 31, 2)]:
        Js = []
        for sgn in (1.0, -1.0):
            s2 = dict(st)
            for k in d:
                s2[k] = st[k] + sgn * h * d[k]
            Js.append(float(objective(run_simulation(s2, mesh, cfg, 1200.0, nsteps=nsteps))))
        fd = (Js[0] - Js[1]) / (2.0 * h)
        rows.append((h, fd, abs(fd - dJ) / abs(dJ)))
    for h, fd, err in rows:
        print(f"terrain FD h=2^{int(round(math.log2(h)))} fd={fd:.12e} adjoint={dJ:.12e} rel_err={err:.3e}")
    assert min(r[2] for r in rows) <= 1e-7, [r[2] for r in rows]
    dJ_u = float((grads["u"].cpu() * d["u"]).sum())
    assert min(abs(fd - dJ_u) / abs(dJ) for _, fd, _ in rows) > 1e-3
