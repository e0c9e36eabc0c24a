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


# ---- derivatives: the reference's own autograd (tests/golden/make_golden_sp_ad.py) ----------
AD = np.load(pathlib.Path(__file__).resolve().parent / "golden" / "sp_ad_g2.npz")
AD_CASES = ("g2_explicit", "g2_moist")
DIFF = ("rho_zz", "qv", "pressure_p", "pressure_base")


@pytest.mark.parametrize("case", AD_CASES)
def test_oracle_derivatives_match_reference_autograd(case):
    from oracle.adjoint import surface_pressure_jvp, surface_pressure_vjp, weighted_sq_sum_vjp
    a = _inputs(case, "step2")
    nc = a["nCells"]
    v = surface_pressure_vjp(nc, a["rho_zz"], a["zz"], a["qv"], a["zgrid"], AD[f"{case}/g_sp"])
    for k in DIFF:
        assert np.array_equal(v[k], AD[f"{case}/grad_{k}"]), k
    t = surface_pressure_jvp(nc, a["rho_zz"], a["zz"], a["qv"], a["zgrid"], *[AD[f"{case}/tan_{k}"] for k in DIFF])
    assert np.array_equal(t, AD[f"{case}/sp_tangent"])
    g = weighted_sq_sum_vjp(AD[f"{case}/sp"][:nc], AD[f"{case}/sp_ref"], AD[f"{case}/area"])
    assert np.array_equal(g, AD[f"{case}/grad_objective_sp"])


def test_mesh_input_derivatives_are_rejected_before_device_work():
    from mpas_dycore_pytorch_gb300.diagnostics import physics_interface_surface_pressure, surface_pressure_functional
    from mpas_dycore_pytorch_gb300.errors import MpasUnsupportedCapabilityError
    z = torch.ones(4, 3, dtype=torch.float64)
    with pytest.raises(MpasUnsupportedCapabilityError, match="zz"):
        physics_interface_surface_pressure(nCells=4, rho_zz=z, zz=z.clone().requires_grad_(True), qv=z,
                                           pressure_p=z, pressure_base=z, zgrid=torch.ones(4, 4, dtype=torch.float64))
    with pytest.raises(MpasUnsupportedCapabilityError, match="area"):
        surface_pressure_functional(z[:, 0], None, torch.ones(4, dtype=torch.float64, requires_grad=True), 4)


def _cuda_inputs(case):
    a = _inputs(case, "step2")
    return a["nCells"], {k: torch.as_tensor(np.ascontiguousarray(v), dtype=torch.float64).cuda()
                         for k, v in a.items() if k != "nCells"}


@pytest.mark.gpu
@pytest.mark.parametrize("case", AD_CASES)
def test_cuda_surface_pressure_derivatives_bit_exact(case):
    """The C-ABI VJP / JVP kernels against the reference's reverse / forward mode."""
    need_gpu()
    import ctypes as C
    from mpas_dycore_pytorch_gb300 import _lib
    lib = _lib.load()
    nc, t = _cuda_inputs(case)
    rows, nlev = t["rho_zz"].shape
    p = lambda x: C.c_void_p(x.data_ptr()) if x is not None else C.c_void_p(0)
    g_sp = torch.as_tensor(AD[f"{case}/g_sp"]).cuda()
    outs = [torch.full((rows, nlev), np.nan, dtype=torch.float64, device="cuda") for _ in DIFF]
    assert lib.mpasg_surface_pressure_vjp(nc, rows, nlev, p(t["rho_zz"]), p(t["zz"]), p(t["qv"]), p(t["zgrid"]),
                                          9.80616, p(g_sp), *[p(o) for o in outs], C.c_void_p(0)) == 0
    for k, o in zip(DIFF, outs):
        assert np.array_equal(o.cpu().numpy(), AD[f"{case}/grad_{k}"]), k
    tan = [torch.as_tensor(AD[f"{case}/tan_{k}"]).cuda() for k in DIFF]
    t_sp = torch.full((rows,), np.nan, dtype=torch.float64, device="cuda")
    assert lib.mpasg_surface_pressure_jvp(nc, rows, nlev, p(t["rho_zz"]), p(t["zz"]), p(t["qv"]), p(t["zgrid"]),
                                          9.80616, *[p(x) for x in tan], p(t_sp), C.c_void_p(0)) == 0
    assert np.array_equal(t_sp.cpu().numpy(), AD[f"{case}/sp_tangent"])
    # a null output is skipped, a null tangent is zero
    assert lib.mpasg_surface_pressure_jvp(nc, rows, nlev, p(t["rho_zz"]), p(t["zz"]), p(t["qv"]), p(t["zgrid"]),
                                          9.80616, None, None, p(tan[2]), None, p(t_sp), C.c_void_p(0)) == 0
    ref = np.concatenate([AD[f"{case}/tan_pressure_p"][:nc, 0], [0.0]])
    assert np.array_equal(t_sp.cpu().numpy(), ref)
    assert lib.mpasg_surface_pressure_vjp(nc, rows + 1, nlev, p(t["rho_zz"]), p(t["zz"]), p(t["qv"]),
                                          p(t["zgrid"]), 9.80616, p(g_sp), None, None, None, None,
                                          C.c_void_p(0)) != 0
    torch.cuda.synchronize()


@pytest.mark.gpu
@pytest.mark.parametrize("case", AD_CASES)
def test_autograd_through_surface_pressure_and_objective(case):
    """torch.autograd.grad / forward_ad through the public functions, as the reference is used."""
    need_gpu()
    import torch.autograd.forward_ad as fwAD
    from mpas_dycore_pytorch_gb300.diagnostics import physics_interface_surface_pressure, surface_pressure_functional
    nc, t = _cuda_inputs(case)
    leaf = {k: (v.clone().requires_grad_(True) if k in DIFF else v) for k, v in t.items()}
    sp = physics_interface_surface_pressure(nCells=nc, **leaf)
    assert np.array_equal(sp.detach().cpu().numpy(), AD[f"{case}/sp"])
    g_sp = torch.as_tensor(AD[f"{case}/g_sp"]).cuda()
    grads = torch.autograd.grad((g_sp * sp).sum(), [leaf[k] for k in DIFF])
    for k, g in zip(DIFF, grads):
        assert np.array_equal(g.cpu().numpy(), AD[f"{case}/grad_{k}"]), k
    with fwAD.dual_level():
        dual = {k: (fwAD.make_dual(v, torch.as_tensor(AD[f"{case}/tan_{k}"]).cuda()) if k in DIFF else v)
                for k, v in t.items()}
        sp_t = fwAD.unpack_dual(physics_interface_surface_pressure(nCells=nc, **dual)).tangent
    assert np.array_equal(sp_t.cpu().numpy(), AD[f"{case}/sp_tangent"])
    # objective: value to 1e-12 (fixed-order tree sum vs torch's), gradient bit-exact
    spl = sp.detach().clone().requires_grad_(True)
    ref = torch.as_tensor(AD[f"{case}/sp_ref"]).cuda()
    area = torch.as_tensor(AD[f"{case}/area"]).cuda()
    obj = surface_pressure_functional(spl, ref, area, nc)
    want = float(AD[f"{case}/objective"])
    assert abs(obj.item() - want) <= 1e-12 * abs(want)
    (g,) = torch.autograd.grad(obj, [spl])
    assert np.array_equal(g[:nc].cpu().numpy(), AD[f"{case}/grad_objective_sp"])
    assert g[nc:].abs().max().item() == 0.0


@pytest.mark.gpu
def test_surface_pressure_jvp_vjp_identity():
    """<g, J t> = <J^T g, t> to 1e-12 on seeded directions, with a failing control."""
    need_gpu()
    import torch.autograd.forward_ad as fwAD
    from mpas_dycore_pytorch_gb300.diagnostics import physics_interface_surface_pressure
    nc, t = _cuda_inputs("g2_moist")
    gen = torch.Generator(device="cuda").manual_seed(11)
    tan = {k: torch.randn(t[k].shape, generator=gen, dtype=torch.float64, device="cuda") for k in DIFF}
    g_sp = torch.randn(t["rho_zz"].shape[0], generator=gen, dtype=torch.float64, device="cuda")
    with fwAD.dual_level():
        dual = {k: (fwAD.make_dual(v, tan[k]) if k in DIFF else v) for k, v in t.items()}
        jt = fwAD.unpack_dual(physics_interface_surface_pressure(nCells=nc, **dual)).tangent
    leaf = {k: (v.clone().requires_grad_(True) if k in DIFF else v) for k, v in t.items()}
    sp = physics_interface_surface_pressure(nCells=nc, **leaf)
    grads = torch.autograd.grad((g_sp * sp).sum(), [leaf[k] for k in DIFF])
    lhs = float((g_sp * jt).sum())
    rhs = float(sum((g * tan[k]).sum() for k, g in zip(DIFF, grads)))
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs))
    bad = rhs + float((grads[0] * tan["rho_zz"]).sum()) * 1e-6  # a perturbed adjoint fails the bound
    assert abs(lhs - bad) > 1e-12 * max(abs(lhs), abs(bad))


def test_dual_mesh_inputs_are_rejected_before_device_work():
    import torch.autograd.forward_ad as fwAD
    from mpas_dycore_pytorch_gb300.diagnostics import physics_interface_surface_pressure
    from mpas_dycore_pytorch_gb300.errors import MpasUnsupportedCapabilityError
    z = torch.ones(4, 3, dtype=torch.float64)
    with fwAD.dual_level():
        zg = fwAD.make_dual(torch.ones(4, 4, dtype=torch.float64), torch.ones(4, 4, dtype=torch.float64))
        with pytest.raises(MpasUnsupportedCapabilityError, match="zgrid"):
            physics_interface_surface_pressure(nCells=4, rho_zz=z, zz=z, qv=z, pressure_p=z, pressure_base=z,
                                               zgrid=zg)


@pytest.mark.gpu
def test_objective_gradient_against_central_differences():
    """Central differences of the area-weighted squared-anomaly objective over
    h = 2^-20 ... 2^-36 in a seeded direction of (rho_zz, qv, pressure_p): the best step
    agrees with <grad, v> from the hand-written VJP chain to 1e-7, and the curve rises
    again at the smallest steps (roundoff), as a central-difference curve does."""
    need_gpu()
    from mpas_dycore_pytorch_gb300.diagnostics import physics_interface_surface_pressure, surface_pressure_functional
    nc, t = _cuda_inputs("g2_moist")
    ref = torch.as_tensor(AD["g2_moist/sp_ref"]).cuda()
    area = torch.as_tensor(AD["g2_moist/area"]).cuda()
    keys = ("rho_zz", "qv", "pressure_p")
    gen = torch.Generator(device="cuda").manual_seed(5)
    # a direction large enough that truncation, not roundoff, limits the largest steps
    scale = {"rho_zz": 1.0, "qv": 0.1, "pressure_p": 1.0e4}
    v = {k: torch.randn(t[k].shape, generator=gen, dtype=torch.float64, device="cuda") * scale[k] for k in keys}

    def objective(h):
        x = dict(t)
        for k in keys:
            x[k] = t[k] + h * v[k]
        return surface_pressure_functional(physics_interface_surface_pressure(nCells=nc, **x), ref, area, nc).item()

    leaf = {k: (val.clone().requires_grad_(True) if k in keys else val) for k, val in t.items()}
    obj = surface_pressure_functional(physics_interface_surface_pressure(nCells=nc, **leaf), ref, area, nc)
    grads = torch.autograd.grad(obj, [leaf[k] for k in keys])
    dot = float(sum((g * v[k]).sum() for k, g in zip(keys, grads)))
    errs = []
    for e in range(20, 37, 2):
        h = 2.0 ** -e
        fd = (objective(h) - objective(-h)) / (2 * h)
        errs.append(abs(fd - dot) / abs(dot))
    assert min(errs) <= 1e-7, errs
    assert errs[-1] > min(errs), errs
