"""Surface-pressure diagnostic: the oracle against the reference's own outputs (CPU),
the CUDA kernel against the same golden vectors (GPU), and the reference's argument
checks."""

import pathlib

import numpy as np
import pytest
import torch

from fixtures import CASES, group, load_case
from gpu_helpers import need_gpu
from oracle.stages import surface_pressure

GOLDEN = np.load(pathlib.Path(__file__).resolve().parent / "golden" / "sp_g2.npz")


def _inputs(case, step):
    meta, st, _ = load_case(case)
    lo, pr, s = group(st, "loaded"), group(st, "prepared"), group(st, step)
    nc = int(np.asarray(lo["nCells"]).reshape(-1)[0])
    return dict(nCells=nc, rho_zz=s["rho_zz"], zz=lo["zz"], qv=np.ascontiguousarray(s["scalars"][..., 0]),
                pressure_p=s["pressure_p"], pressure_base=pr["pressure_base"], zgrid=lo["zgrid"])


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("step", ("step1", "step2"))
def test_oracle_matches_reference_bit_for_bit(case, step):
    a = _inputs(case, step)
    got = surface_pressure(**a)
    assert np.array_equal(got, GOLDEN[f"{case}/{step}"])


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("step", ("step1", "step2"))
def test_cuda_surface_pressure_bit_exact(case, step):
    need_gpu()
    from mpas_dycore_pytorch_gb300.diagnostics import physics_interface_surface_pressure
    a = _inputs(case, step)
    t = {k: (torch.as_tensor(v, dtype=torch.float64).cuda() if isinstance(v, np.ndarray) else v) for k, v in a.items()}
    got = physics_interface_surface_pressure(**t).cpu().numpy()
    assert np.array_equal(got, GOLDEN[f"{case}/{step}"])
    # active rows only: no padding row in the output
    t2 = {k: (v[:a["nCells"]] if isinstance(v, torch.Tensor) else v) for k, v in t.items()}
    assert np.array_equal(physics_interface_surface_pressure(**t2).cpu().numpy(), GOLDEN[f"{case}/{step}"][:-1])


@pytest.mark.gpu
def test_functional_is_deterministic_and_matches_numpy():
    need_gpu()
    from mpas_dycore_pytorch_gb300.diagnostics import surface_pressure_functional
    g = torch.Generator().manual_seed(3)
    x = torch.rand(40963, generator=g, dtype=torch.float64) * 1e5
    r = torch.rand(40963, generator=g, dtype=torch.float64) * 1e5
    w = torch.rand(40963, generator=g, dtype=torch.float64)
    a = surface_pressure_functional(x.cuda(), r.cuda(), w.cuda(), 40962)
    b = surface_pressure_functional(x.cuda(), r.cuda(), w.cuda(), 40962)
    assert a.item() == b.item()
    ref = float(np.sum(w.numpy()[:40962] * (x.numpy()[:40962] - r.numpy()[:40962]) ** 2))
    assert abs(a.item() - ref) <= 1e-12 * abs(ref)


def test_argument_checks_follow_the_reference():
    from mpas_dycore_pytorch_gb300.diagnostics import physics_interface_surface_pressure
    z = torch.zeros(4, 3, dtype=torch.float64)
    with pytest.raises(ValueError, match="must be rank-2"):
        physics_interface_surface_pressure(nCells=4, rho_zz=torch.zeros(4), zz=z, qv=z, pressure_p=z,
                                           pressure_base=z, zgrid=torch.zeros(4, 4))
    with pytest.raises(ValueError, match="first dimension must be nCells"):
        physics_interface_surface_pressure(nCells=2, rho_zz=z, zz=z, qv=z, pressure_p=z, pressure_base=z,
                                           zgrid=torch.zeros(4, 4))
