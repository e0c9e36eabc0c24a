"""Tridiagonal solve / factorisation derivatives.

CPU: the oracle against the reference's own forward, reverse-mode and forward-mode
outputs (golden ``tridiag_ref.npz``).  GPU: the CUDA Functions against the same vectors,
the reference's JVP/VJP identity test (tests/test_derivative_identity.py of the
reference, bound 8 n eps / (1 - n eps)) with its failing control, and the identity on a
40962-column system."""

import pathlib

import numpy as np
import pytest
import torch

from gpu_helpers import need_gpu
from oracle import adjoint as A

G = np.load(pathlib.Path(__file__).resolve().parent / "golden" / "tridiag_ref.npz")
TAGS = ("3x6", "17x41")


def _g(tag, name):
    return G[f"{tag}/{name}"]


def _rel(x, y):
    return np.linalg.norm((x - y).ravel()) / max(np.linalg.norm(y.ravel()), 1e-300)


@pytest.mark.parametrize("tag", TAGS)
def test_oracle_matches_reference(tag):
    a, b, c, rhs = (_g(tag, k) for k in ("a", "b", "c", "rhs"))
    al, ga = A.factor(a, b, c)
    assert _rel(al, _g(tag, "alpha")) < 1e-15 and _rel(ga, _g(tag, "gamma")) < 1e-15
    al, ga = _g(tag, "alpha"), _g(tag, "gamma")
    out = A.solve(a, al, ga, rhs)
    assert _rel(out, _g(tag, "out")) < 1e-14
    vjp = A.solve_vjp(a, al, ga, rhs, _g(tag, "out"), _g(tag, "solve_w"))
    for nm, v in zip(("a", "alpha", "gamma", "rhs"), vjp):
        assert _rel(v, _g(tag, f"solve_vjp_{nm}")) < 1e-13, nm
    tans = [_g(tag, f"solve_tan_{nm}") for nm in ("a", "alpha", "gamma", "rhs")]
    assert _rel(A.solve_jvp(a, al, ga, rhs, _g(tag, "out"), *tans), _g(tag, "solve_jvp")) < 1e-13
    fv = A.factor_vjp(a, c, al, ga, _g(tag, "factor_wa"), _g(tag, "factor_wg"))
    for nm, v in zip(("a", "b", "c"), fv):
        assert _rel(v, _g(tag, f"factor_vjp_{nm}")) < 1e-13, nm
    ft = [_g(tag, f"factor_tan_{nm}") for nm in ("a", "b", "c")]
    dal, dga = A.factor_jvp(a, c, al, ga, *ft)
    assert _rel(dal, _g(tag, "factor_jvp_alpha")) < 1e-13 and _rel(dga, _g(tag, "factor_jvp_gamma")) < 1e-13


def _cuda(x):
    return torch.as_tensor(np.asarray(x), dtype=torch.float64).cuda()


@pytest.mark.gpu
@pytest.mark.parametrize("tag", TAGS)
def test_cuda_functions_match_reference(tag):
    need_gpu()
    import torch.autograd.forward_ad as fw
    from mpas_dycore_pytorch_gb300.autodiff import TridiagonalFactorize, TridiagonalSolve
    a, b, c, rhs = (_cuda(_g(tag, k)) for k in ("a", "b", "c", "rhs"))
    al, ga = TridiagonalFactorize.apply(a, b, c)
    assert _rel(al.cpu().numpy(), _g(tag, "alpha")) < 1e-14
    assert _rel(ga.cpu().numpy(), _g(tag, "gamma")) < 1e-14
    al, ga = _cuda(_g(tag, "alpha")), _cuda(_g(tag, "gamma"))
    out = TridiagonalSolve.apply(a, al, ga, rhs)
    assert _rel(out.cpu().numpy(), _g(tag, "out")) < 1e-14
    ins = [t.clone().requires_grad_(True) for t in (a, al, ga, rhs)]
    grads = torch.autograd.grad((TridiagonalSolve.apply(*ins) * _cuda(_g(tag, "solve_w"))).sum(), ins)
    for nm, v in zip(("a", "alpha", "gamma", "rhs"), grads):
        assert _rel(v.cpu().numpy(), _g(tag, f"solve_vjp_{nm}")) < 1e-13, nm
    tans = [_cuda(_g(tag, f"solve_tan_{nm}")) for nm in ("a", "alpha", "gamma", "rhs")]
    with fw.dual_level():
        duals = [fw.make_dual(p, t) for p, t in zip((a, al, ga, rhs), tans)]
        tout = fw.unpack_dual(TridiagonalSolve.apply(*duals))[1]
    assert _rel(tout.cpu().numpy(), _g(tag, "solve_jvp")) < 1e-13
    fins = [t.clone().requires_grad_(True) for t in (a, b, c)]
    fal, fga = TridiagonalFactorize.apply(*fins)
    fg = torch.autograd.grad((fal * _cuda(_g(tag, "factor_wa"))).sum() + (fga * _cuda(_g(tag, "factor_wg"))).sum(),
                             fins)
    for nm, v in zip(("a", "b", "c"), fg):
        assert _rel(v.cpu().numpy(), _g(tag, f"factor_vjp_{nm}")) < 1e-13, nm
    ft = [_cuda(_g(tag, f"factor_tan_{nm}")) for nm in ("a", "b", "c")]
    with fw.dual_level():
        o1, o2 = TridiagonalFactorize.apply(*[fw.make_dual(p, t) for p, t in zip((a, b, c), ft)])
        d1, d2 = fw.unpack_dual(o1)[1], fw.unpack_dual(o2)[1]
    assert _rel(d1.cpu().numpy(), _g(tag, "factor_jvp_alpha")) < 1e-13
    assert _rel(d2.cpu().numpy(), _g(tag, "factor_jvp_gamma")) < 1e-13


def _identity_residual(jvp, weight, direction, vjp):
    left, right = (jvp.reshape(-1) * weight.reshape(-1)), (direction.reshape(-1) * vjp.reshape(-1))
    lhs, rhs = torch.sum(left, dtype=torch.float64), torch.sum(right, dtype=torch.float64)
    den = max(float((torch.sum(torch.abs(left)) + torch.sum(torch.abs(right))).item()),
              torch.finfo(torch.float64).tiny)
    n = max(left.numel(), right.numel())
    eps = torch.finfo(torch.float64).eps
    return abs(float((lhs - rhs).item())) / den, 8.0 * (n * eps / (1.0 - n * eps))


@pytest.mark.gpu
@pytest.mark.parametrize("shape", ((1, 4), (40962, 55)))
def test_jvp_vjp_identity_and_failing_control(shape):
    """The reference's identity check (its 1x4 system and a full-size column set)."""
    need_gpu()
    import torch.autograd.forward_ad as fw
    from mpas_dycore_pytorch_gb300.autodiff import TridiagonalSolve
    n, L = shape
    if shape == (1, 4):
        a = torch.tensor([[0.0, 0.08, -0.05, 0.03]], dtype=torch.float64)
        alpha = torch.tensor([[1.0, 0.95, 1.03, 0.98]], dtype=torch.float64)
        gamma = torch.tensor([[0.04, -0.02, 0.06, 0.01]], dtype=torch.float64)
        primal = torch.tensor([[1.0, -0.5, 0.75, 0.2, -0.1]], dtype=torch.float64)
    else:
        g = torch.Generator().manual_seed(11)
        a = 0.05 * torch.randn(n, L, generator=g, dtype=torch.float64)
        alpha = 1.0 + 0.05 * torch.randn(n, L, generator=g, dtype=torch.float64)
        gamma = 0.05 * torch.randn(n, L, generator=g, dtype=torch.float64)
        primal = torch.randn(n, L + 1, generator=g, dtype=torch.float64)
    direction = torch.randn(primal.shape, dtype=torch.float64, generator=torch.Generator().manual_seed(7301))
    weight = torch.randn(primal.shape, dtype=torch.float64, generator=torch.Generator().manual_seed(9109))
    a, alpha, gamma, primal, direction, weight = (t.cuda() for t in (a, alpha, gamma, primal, direction, weight))
    with fw.dual_level():
        jvp = fw.unpack_dual(TridiagonalSolve.apply(a, alpha, gamma, fw.make_dual(primal, direction)))[1]
    rhs = primal.clone().requires_grad_(True)
    vjp = torch.autograd.grad(torch.sum(TridiagonalSolve.apply(a, alpha, gamma, rhs) * weight, dtype=torch.float64),
                              rhs)[0]
    res, bound = _identity_residual(jvp, weight, direction, vjp)
    assert res <= bound, (res, bound)
    control, _ = _identity_residual(jvp, weight, direction, torch.zeros_like(vjp))
    assert control > 1.0e-6
