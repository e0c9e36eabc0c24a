"""CUDA step vs the CPU oracle on a 2562-cell x 26-level mesh (the CPU-runnable config),
and size-independent properties on a larger mesh."""

import numpy as np
import pytest
import torch

from fixtures import rel_l2
from gpu_helpers import need_gpu, to_np

pytestmark = pytest.mark.gpu

CFG0 = {"config_time_integration_order": 3, "config_len_disp": 120000.0, "config_monotonic": False,
        "config_dt": 1800.0}


OPTIONS = {"config_horiz_mixing": "2d_fixed", "config_h_mom_eddy_visc4": 1.0e10,
           "config_h_theta_eddy_visc4": 5.0e9, "config_h_theta_eddy_visc2": 2.0e4,
           "config_v_mom_eddy_visc2": 1.0, "config_v_theta_eddy_visc2": 1.0,
           "config_mpas_cam_coef": 1.0, "config_apvm_upwinding": 1.0}


def _case(level, nlev, ntr, mono, seed=0, dz=None, options=None):
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.loader import load_case
    cfg = dict(CFG0)
    cfg["config_monotonic"] = mono
    cfg.update(options or {})
    spec = CaseSpec(level=level, nlev=nlev, seed=seed, n_bumps=8, n_tracers=ntr, dz_bottom=dz)
    st, _ = load_case(spec, cfg, as_torch=False)
    return st, cfg


@pytest.mark.parametrize("mono,options", [(False, None), (True, None), (True, OPTIONS)],
                         ids=["explicit", "monotone", "monotone_mixing_options"])
def test_level4_two_steps_vs_oracle(mono, options):
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import Model
    from oracle.step import Stepper
    st, cfg = _case(4, 26, 3 if mono else 1, mono, options=options)
    model = Model(st, cfg, 1800.0, num_scalars=st["scalars"].shape[-1])
    model.prepare(st)
    ref = Stepper(st, cfg)
    rs = ref.prepare(st, 1800.0)
    for _ in range(2):
        model.step()
        rs = ref.srk3_step(rs, 1800.0)
    got = model.export()
    for k in ("u", "w", "theta_m", "rho_zz", "scalars", "exner", "pressure_p", "v", "vorticity",
              "divergence", "ke", "pv_edge", "uReconstructZonal", "ruAvg", "wwAvg"):
        err = rel_l2(to_np(got[k])[:-1], rs[k][:-1])
        assert err <= 1e-12, (k, err)


def test_monotone_tracers_stay_bounded_level5():
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import Model
    st, cfg = _case(5, 20, 3, True, seed=2, dz=200.0)
    model = Model(st, cfg, 900.0, num_scalars=3)
    model.prepare(st)
    q0 = to_np(model.state.f["scalars"])[:-1].copy()
    for _ in range(3):
        model.step()
    q = to_np(model.state.f["scalars"])[:-1]
    assert np.isfinite(q).all()
    assert q.min() >= -1e-14
    assert q.max() <= q0.max() * (1 + 1e-10) + 1e-12
    assert model.check_finite() == 0


def test_no_scalars_two_steps_vs_oracle():
    """An empty scalar set (num_scalars = 0): the dynamics alone, against the oracle."""
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import Model
    from oracle.step import Stepper
    st, cfg = _case(3, 16, 0, False)
    assert st["scalars"].shape[-1] == 0
    model = Model(st, cfg, 1800.0, num_scalars=0)
    model.prepare(st)
    ref = Stepper(st, cfg)
    rs = ref.prepare(st, 1800.0)
    for _ in range(2):
        model.step()
        rs = ref.srk3_step(rs, 1800.0)
    got = model.export()
    for k in ("u", "w", "theta_m", "rho_zz", "exner", "v", "divergence", "uReconstructZonal"):
        err = rel_l2(to_np(got[k])[:-1], rs[k][:-1])
        assert err <= 1e-12, (k, err)
    assert model.check_finite() == 0
