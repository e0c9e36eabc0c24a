"""Batched ensemble on the GPU: each member of a union of uneven meshes gives exactly
the result of running that member alone (float64 and mixed forms)."""

import pytest
import torch

from gpu_helpers import need_gpu

pytestmark = pytest.mark.gpu

CFG = {"config_time_integration_order": 3, "config_len_disp": 120000.0, "config_number_of_sub_steps": 2,
       "config_dynamics_split_steps": 3, "config_monotonic": True, "config_dt": 600.0}


@pytest.fixture(scope="module")
def members():
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.ensemble import member_cases
    from mpas_dycore_pytorch_gb300.loader import load_case
    a = member_cases(CaseSpec(level=3, nlev=16, n_bumps=3, n_tracers=2), seeds=[10, 11], config=CFG, u_noise=0.5)
    b, _ = load_case(CaseSpec(level=2, nlev=16, seed=12, n_bumps=2, n_tracers=2), CFG, as_torch=False)
    return a + [b]


@pytest.mark.parametrize("precision", ("float64", "mixed"))
def test_members_match_individual_runs(members, precision):
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import Model
    from mpas_dycore_pytorch_gb300.device import STATE_KEYS
    from mpas_dycore_pytorch_gb300.ensemble import Ensemble
    ens = Ensemble(members, CFG, 600.0, precision=precision)
    for _ in range(2):
        ens.step()
    torch.cuda.synchronize()
    for b, m in enumerate(members):
        solo = Model(m, CFG, 600.0, num_scalars=2, precision=precision)
        solo.prepare(m)
        for _ in range(2):
            solo.step()
        got = ens.member_state(b)
        for k in STATE_KEYS:
            want = solo.state.f[k][:-1]
            assert torch.equal(got[k][:-1], want), (precision, b, k)


@pytest.mark.parametrize("precision", ("float64", "mixed"))
def test_groups_on_different_vertical_grids_in_one_graph(members, precision):
    """Members on two vertical grids (16 and 12 levels) with different timesteps: one CUDA
    graph replays both groups' steps, and every member matches its solo run bit for bit."""
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import Model
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.device import STATE_KEYS
    from mpas_dycore_pytorch_gb300.ensemble import EnsembleGroups, member_cases
    cfg12 = dict(CFG, config_dt=900.0, config_monotonic=False)
    other = member_cases(CaseSpec(level=3, nlev=12, n_bumps=2, n_tracers=2, dz_bottom=300.0), seeds=[20, 21, 22],
                         config=cfg12, u_noise=0.5)
    groups = [(members, CFG, 600.0), (other, cfg12, 900.0)]
    ens = EnsembleGroups(groups, precision=precision)
    ens.capture_graph()
    for _ in range(2):
        ens.step()
    torch.cuda.synchronize()
    assert ens.check_finite() == 0
    for gi, (mems, cfg, dt) in enumerate(groups):
        for b, m in enumerate(mems):
            solo = Model(m, cfg, dt, num_scalars=2, precision=precision)
            solo.prepare(m)
            for _ in range(2):
                solo.step()
            got = ens.member_state(gi, b)
            for k in STATE_KEYS:
                assert torch.equal(got[k][:-1], solo.state.f[k][:-1]), (precision, gi, b, k)
