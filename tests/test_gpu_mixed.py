"""Mixed form (float32 stencils over float64 state) against the float64 form.

The stated accuracy of the mixed form: every state field within relative L2 1e-5 of the
float64 form after 24 large steps (the reference's float64 arithmetic is what the float64
form reproduces to 1e-12, see test_gpu_step.py).  Also checks the mixed form's integer
float64<->float32 conversion and Newton-Raphson reciprocal against CUDA's own conversion
and division.
"""

import ctypes as C

import numpy as np
import pytest
import torch

from gpu_helpers import need_gpu

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-5  # per-field relative L2 after 24 steps
STEPS = 24


def _numerics(which, x):
    from mpas_dycore_pytorch_gb300 import _lib
    lib = _lib.load()
    out = torch.empty_like(x)
    rc = lib.mpasg_numerics_check(which, C.c_void_p(x.data_ptr()), C.c_void_p(out.data_ptr()), x.numel(),
                                  C.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc, "mpasg_numerics_check")
    torch.cuda.synchronize()
    return out


def _samples(n=200_000, seed=0):
    g = torch.Generator().manual_seed(seed)
    mant = torch.rand(n, generator=g, dtype=torch.float64) + 0.5
    expo = torch.randint(-120, 120, (n,), generator=g).to(torch.float64)
    sign = torch.where(torch.rand(n, generator=g) < 0.5, -1.0, 1.0).to(torch.float64)
    return (sign * mant * torch.pow(2.0, expo)).cuda()


def test_float32_repacking_matches_cuda_conversion():
    need_gpu()
    x = _samples()
    got = _numerics(0, x)
    ref = x.float().double()  # CUDA's round-to-nearest-even conversion
    assert torch.all(torch.abs(got - x) <= torch.abs(x) * 2.0 ** -24)
    # ties (round half away vs half even) are the only possible differences
    assert (got == ref).double().mean().item() > 0.9999
    z = torch.zeros(4, dtype=torch.float64, device="cuda")
    assert torch.equal(_numerics(0, z), z)


def test_newton_reciprocal_within_two_ulp():
    need_gpu()
    x = _samples(seed=1)
    got = _numerics(1, x)
    ref = 1.0 / x  # CUDA's correctly rounded float64 division
    assert torch.all(torch.abs(got - ref) <= 2.0 * 2.0 ** -52 * torch.abs(ref))


def _run(case_spec, cfg, dt, precision, steps):
    from mpas_dycore_pytorch_gb300.api import Model
    from mpas_dycore_pytorch_gb300.device import STATE_KEYS
    from mpas_dycore_pytorch_gb300.loader import load_case
    st, _ = load_case(case_spec, cfg, as_torch=False)
    model = Model(st, cfg, dt, num_scalars=int(st["scalars"].shape[-1]), precision=precision)
    model.prepare(st)
    for _ in range(steps):
        model.step()
    assert model.check_finite() == 0
    return {k: model.state.f[k][:-1].cpu().numpy() for k in STATE_KEYS}


def test_mixed_form_within_stated_error_after_24_steps():
    need_gpu()
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    # level-5 mesh (10242 cells), 41 levels, 3 monotone tracers
    spec = CaseSpec(level=5, nlev=41, seed=2, n_bumps=8, n_tracers=3)
    cfg = {"config_time_integration_order": 3, "config_len_disp": 120000.0, "config_number_of_sub_steps": 2,
           "config_dynamics_split_steps": 3, "config_monotonic": True, "config_dt": 900.0}
    ref = _run(spec, cfg, 900.0, "float64", STEPS)
    got = _run(spec, cfg, 900.0, "mixed", STEPS)
    worst = {}
    for k, r in ref.items():
        den = np.linalg.norm(r.ravel())
        if den == 0.0:
            assert np.array_equal(got[k], r), k
            continue
        worst[k] = float(np.linalg.norm((got[k] - r).ravel()) / den)
    bad = {k: v for k, v in worst.items() if v > MIXED_TOL}
    assert not bad, bad
    # the mixed form really differs from the float64 form (float32 arithmetic ran)
    assert max(worst.values()) > 1e-12


@pytest.mark.parametrize("options", [
    {"config_horiz_mixing": "2d_fixed", "config_h_mom_eddy_visc4": 1.0e10, "config_h_theta_eddy_visc4": 5.0e9,
     "config_h_theta_eddy_visc2": 2.0e4, "config_v_mom_eddy_visc2": 1.0, "config_v_theta_eddy_visc2": 1.0},
    {"config_mpas_cam_coef": 1.0, "config_number_cam_damping_levels": 4, "config_apvm_upwinding": 1.0},
    {"config_rayleigh_damp_u": True, "config_rayleigh_damp_u_timescale_days": 0.5,
     "config_number_rayleigh_damp_u_levels": 6, "config_mix_full": False, "config_v_mom_eddy_visc2": 2.0,
     "config_v_theta_eddy_visc2": 2.0},
], ids=["fixed_vertical_mixing", "cam_damping", "rayleigh_perturbation_mixing"])
def test_mixed_form_with_mixing_options(options):
    """The mixing options (2d_fixed, vertical mixing, CAM damping) in the mixed form stay
    within the stated error of the float64 form (6 steps on the level-4 mesh)."""
    need_gpu()
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    spec = CaseSpec(level=4, nlev=26, seed=4, n_bumps=8, n_tracers=1, w_sine=0.05)
    cfg = {"config_time_integration_order": 3, "config_len_disp": 240000.0, "config_number_of_sub_steps": 2,
           "config_dynamics_split_steps": 3, "config_monotonic": True, "config_dt": 1200.0}
    cfg.update(options)
    ref = _run(spec, cfg, 1200.0, "float64", 6)
    got = _run(spec, cfg, 1200.0, "mixed", 6)
    worst = {}
    for k, r in ref.items():
        den = np.linalg.norm(r.ravel())
        if den > 0.0:
            worst[k] = float(np.linalg.norm((got[k] - r).ravel()) / den)
    bad = {k: v for k, v in worst.items() if v > MIXED_TOL}
    assert not bad, bad
    assert max(worst.values()) > 1e-12


def test_mixed_form_over_terrain():
    """Terrain-following levels over a 1500 m cosine hill (the slope terms of the small-step
    perturbation, the recovery of w and the u tendency's zxu term in their float32 forms)
    stay within the stated error of the float64 form (6 steps on the level-4 mesh)."""
    need_gpu()
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    spec = CaseSpec(level=4, nlev=26, dz_bottom=300.0, seed=6, n_bumps=8, n_tracers=1, w_sine=0.05,
                    terrain=1500.0)
    cfg = {"config_time_integration_order": 3, "config_len_disp": 240000.0, "config_number_of_sub_steps": 2,
           "config_dynamics_split_steps": 3, "config_monotonic": True, "config_dt": 1200.0}
    ref = _run(spec, cfg, 1200.0, "float64", 6)
    got = _run(spec, cfg, 1200.0, "mixed", 6)
    worst = {}
    for k, r in ref.items():
        den = np.linalg.norm(r.ravel())
        if den > 0.0:
            worst[k] = float(np.linalg.norm((got[k] - r).ravel()) / den)
    print({k: f"{v:.2e}" for k, v in sorted(worst.items(), key=lambda kv: -kv[1])[:4]})
    bad = {k: v for k, v in worst.items() if v > MIXED_TOL}
    assert not bad, bad
    assert max(worst.values()) > 1e-12
