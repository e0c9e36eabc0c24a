"""The hand-written reverse mode of the dynamics on the GPU.

* every stage's CUDA VJP against the oracle's stage VJP (oracle/dyn_adjoint.py, itself pinned
  to the reference's autograd) on the reference's own stage calls (golden taps), with seeded
  output cotangents;
* run_simulation.vjp of the area-weighted squared surface-pressure anomaly with respect to
  the loaded u and theta against the gradients the reference computed
  (tests/golden/make_golden_dyn_ad.py), within the stated 1e-10.
"""

import ctypes as C

import numpy as np
import pytest
import torch

import oracle.dyn_adjoint as D
from dyn_ad_fixtures import AD_CASES, AD_OPTION_CASES, AD_TERRAIN_CASES, _npz, config, mesh_and_state
from fixtures import tap_calls
from gpu_helpers import model_for_case, need_gpu, to_np
from oracle.step import stage_names

pytestmark = pytest.mark.gpu

PRE = "_vertical_implicit_coefficients_"
# dry cases whose options the derivative covers
STAGE_CASES = ("g2_explicit", "g2_mono", "g2_rk2", "g2_split2", "g2_fixed", "g2_cam", "g2_rayleigh", "g2_terrain")
# per stage: the C entry point's scalar arguments, the output cotangents seeded (reference
# names) and the inputs compared (reference names)
STAGE_SPEC = {
    "vimp": ([PRE + k for k in ("cofwz_active", "coftz_active", "cofwt_active", "a_tri_active", "alpha_tri_active",
                                "gamma_tri_active")], ["p", "t", "rt"]),
    "dyn_tend": (["tend_u", "tend_w", "tend_theta", "tend_rho", "tend_u_euler", "tend_w_euler", "tend_theta_euler"],
                 ["u", "v", "w", "ru", "rw", "ru_save", "rw_save", "theta_m", "theta_m_save", "rho_zz", "rho_edge",
                  "divergence", "vorticity", "ke", "pv_edge", "pp", "rr_save", "tend_rho_in", "tend_u_euler_in",
                  "tend_w_euler_in", "tend_theta_euler_in"]),
    "smlstep": (["w_tend"], ["w_tend", "u_tend"]),
    "acoustic": (["ru_p", "rho_pp", "rtheta_pp", "rtheta_pp_old", "rw_p"],
                 ["ru_p", "rho_pp", "rtheta_pp", "rw_p", "tend_ru", "tend_rho", "tend_rt", "tend_rw", "exner",
                  "theta_m", "rho_zz", "w", "rw", "rw_save"] +
                 [PRE + k for k in ("cofwz_active", "coftz_active", "cofwt_active", "a_tri_active",
                                    "alpha_tri_active", "gamma_tri_active")]),
    "divdamp": (["ru_p"], ["ru_p", "rtheta_pp", "rtheta_pp_old", "theta_m"]),
    "recover": (["rho_p", "rho_zz", "rtheta_p", "theta_m", "u", "ru", "w", "rw", "exner", "pressure_p"],
                ["rho_p_save", "rho_pp", "rtheta_p_save", "rtheta_pp", "rw_save", "rw_p", "ru_save", "ru_p"]),
    "diag": (["h_edge", "v", "divergence", "vorticity", "ke", "pv_edge"], ["u", "h", "v_in"]),
}
ORACLE = {"vimp": D.vimp_vjp, "dyn_tend": D.dyn_tend_vjp, "smlstep": D.smlstep_vjp, "acoustic": D.acoustic_vjp,
          "divdamp": D.divdamp_vjp, "recover": D.recover_vjp, "diag": D.diag_vjp}
# edge-sum cotangent of theta_m_save: the CUDA reverse keeps the part that flows through the
# edge mean per edge (gathered on the cells at the substep start); theta_m / theta_m_save
# inputs of these stages compare after that gather
EDGE_SUM_INPUT = {"acoustic": "theta_m", "divdamp": "theta_m", "dyn_tend": "theta_m_save"}


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _call(model, adj, key, inp):
    lib, m, c = model.lib, C.byref(model.dmesh.struct), C.byref(model.cstruct)
    f, g, t, w = C.byref(model.state.struct), C.byref(adj.g.struct), C.byref(adj.t), C.c_void_p(adj.work.data_ptr())
    s = _stream()
    if key == "vimp":
        rc = lib.mpasg_vert_imp_coefs(m, c, f, float(inp["dts"]), s)
        assert rc == 0
        return lib.mpasg_vimp_vjp(m, c, f, g, float(inp["dts"]), w, s)
    if key == "dyn_tend":
        return lib.mpasg_dyn_tend_vjp(m, c, f, g, t, int(inp["rk_step"]), w, s)
    if key == "smlstep":
        return lib.mpasg_smlstep_vjp(m, c, f, g, s)
    if key == "acoustic":
        return lib.mpasg_acoustic_vjp(m, c, f, g, t, int(inp["small_step"]), float(inp["dts"]), w, s)
    if key == "divdamp":
        return lib.mpasg_divdamp_vjp(m, c, f, g, float(inp["dts"]), w, s)
    if key == "recover":
        return lib.mpasg_recover_vjp(m, c, f, g, int(inp["rk_step"]), int(inp["ns"]), float(inp["dt"]), w, s)
    return lib.mpasg_diag_vjp(m, c, f, g, t, int(inp["rk_step"]), w, s)


def _edge_sum_to_cells(model, ge):
    """theta_m_save's cotangent from the per-edge edge-sum cotangent: each cell collects its edges."""
    dm = model.dmesh
    nc, L = dm.nCells, dm.nVertLevels
    eoc = torch.as_tensor(np.asarray(dm.ints["edgesOnCell"], dtype=np.int64), device=ge.device)
    n = torch.as_tensor(np.asarray(dm.ints["nEdgesOnCell"], dtype=np.int64), device=ge.device)
    out = torch.zeros((nc + 1, L), dtype=torch.float64, device=ge.device)
    for j in range(eoc.shape[1]):
        ok = (j < n)
        e = torch.where(ok, eoc[:, j], torch.full_like(eoc[:, j], dm.nEdges))
        out[:nc] += torch.where(ok[:, None], ge[e], torch.zeros_like(ge[e]))
    return out


@pytest.mark.parametrize("case", STAGE_CASES)
@pytest.mark.parametrize("key", sorted(STAGE_SPEC))
def test_stage_vjp_matches_oracle(case, key):
    need_gpu()
    from mpas_dycore_pytorch_gb300.dyn_adjoint import DynamicsAdjoint
    from mpas_dycore_pytorch_gb300.stages import STAGES
    calls = [call for name in stage_names(key) for call in tap_calls(case, name)]
    if not calls:
        pytest.skip("stage not called in this case")
    model, _, _, _ = model_for_case(case)
    adj = DynamicsAdjoint(model)
    _, _, ins, outs = STAGES[key]
    seed_outs, compare = STAGE_SPEC[key]
    for ci, (inp, _out, entry) in enumerate(calls):
        st = model.state
        for ref_name, field in ins.items():
            if hasattr(inp.get(ref_name), "shape"):
                st.load({field: inp[ref_name]}, keys=(field,))
        adj.zero_cotangents()
        rng = np.random.default_rng(500 + ci)
        gout = {}
        nrows = {int(inp.get("nCells", -9)), int(inp.get("nEdges", -9)), int(inp.get("nVertices", -9))}
        for name in seed_outs:
            field = outs.get(name, name)
            if name in ("exner", "pressure_p") and key == "recover" and int(inp["rk_step"]) != 3:
                continue
            shape = tuple(st.f[field].shape)
            gg = rng.standard_normal(shape)
            if shape[0] - 1 in nrows:
                gg[-1] = 0.0
            # the oracle takes the reference's shapes (the coefficients have active rows only)
            ref_rows = np.asarray(_out[name]).shape[0] if name in _out else shape[0]
            gout[name] = gg[:ref_rows]
            adj.g.f[field].copy_(torch.as_tensor(gg))
        want = ORACLE[key](inp, gout)
        rc = _call(model, adj, key, inp)
        assert rc == 0, (key, rc)
        torch.cuda.synchronize()
        for name in compare:
            if name not in want:
                continue
            field = ins[name]
            got = adj.g.f[field].clone()
            if EDGE_SUM_INPUT.get(key) == name:
                got = got + _edge_sum_to_cells(model, adj.g.f["theta_edge_save"])
            w = np.asarray(want[name])
            got = to_np(got)
            if w.shape != got.shape:
                got = got[: w.shape[0]]
            rows = w.shape[0] - 1 if (w.shape[0] - 1) in nrows else w.shape[0]
            den = np.linalg.norm(w[:rows])
            err = np.linalg.norm(got[:rows] - w[:rows]) / (den if den > 0 else 1.0)
            assert err <= 1e-12, (key, entry["index"], name, err, den)


def _reference_objective(model_mesh, sp_ref, nc):
    from mpas_dycore_pytorch_gb300.diagnostics import physics_interface_surface_pressure, surface_pressure_functional
    dev = torch.device("cuda")
    zz = torch.as_tensor(np.asarray(model_mesh["zz"]), dtype=torch.float64, device=dev)
    zgrid = torch.as_tensor(np.asarray(model_mesh["zgrid"]), dtype=torch.float64, device=dev)
    area = torch.as_tensor(np.asarray(model_mesh["areaCell"]), dtype=torch.float64, device=dev)
    ref = torch.as_tensor(sp_ref, dtype=torch.float64, device=dev)

    def objective(out):
        rz = out["rho_zz"]
        sp = physics_interface_surface_pressure(nCells=nc, rho_zz=rz, zz=zz, qv=torch.zeros_like(rz),
                                                pressure_p=out["pressure_p"],
                                                pressure_base=out["pressure_base"].to(dev), zgrid=zgrid)
        return surface_pressure_functional(sp, ref, area, nc)

    return objective


@pytest.mark.parametrize("case", AD_CASES + AD_OPTION_CASES + AD_TERRAIN_CASES)
def test_run_vjp_matches_reference(case):
    """run_simulation.vjp(track_keys=("u", "theta")) of the surface-pressure functional, against
    the reference's run_simulation.vjp on the same inputs: rel L2 <= 1e-10 or, where larger,
    the gradient's own conditioning (its change when u and theta move by one unit in the last
    place): the Smagorinsky coefficient of a nearly rigid flow is the square root of a
    deformation made of roundoff, so the u gradient's share through it follows the roundings
    of the forward run (at fixed-coefficient mixing, flat or over terrain, the gradients
    agree to ~1e-13)."""
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import run_simulation
    z = _npz(case)
    mesh, st0 = mesh_and_state(case)
    nc = int(mesh["nCells"])
    objective = _reference_objective(mesh, z["sp_ref"], nc)
    state = {k: torch.as_tensor(v) for k, v in st0.items()}
    kw = dict(track_keys=("u", "theta"), config=config(case), dt=float(z["dt"]), nsteps=int(z["nsteps"]))
    grads = run_simulation.vjp(state, mesh, objective, **kw)
    rng = np.random.default_rng(5)
    noisy = dict(state)
    for key in ("u", "theta"):
        x = state[key].numpy().copy()
        x[:-1] *= 1.0 + 2.0 ** -52 * rng.choice([-1.0, 0.0, 1.0], size=x[:-1].shape)
        noisy[key] = torch.as_tensor(x)
    grads_n = run_simulation.vjp(noisy, mesh, objective, **kw)
    for k in ("u", "theta"):
        a = to_np(grads[k])[:-1]
        b = z[f"grad_{k}"][:-1]
        err = np.linalg.norm(a - b) / np.linalg.norm(b)
        floor = np.linalg.norm(to_np(grads_n[k])[:-1] - a) / np.linalg.norm(a)
        print(f"{case} grad_{k}: rel L2 vs reference {err:.3e} (1-ulp input conditioning {floor:.3e})")
        assert err <= max(1e-10, floor), (case, k, err, floor)
    # without the per-step checkpoint (every step's tape kept, nothing recomputed) the
    # reverse pass reads the same tapes: the same gradients bit for bit
    state = {k: torch.as_tensor(v) for k, v in st0.items()}
    again = run_simulation.vjp(state, mesh, objective, track_keys=("u", "theta"), config=config(case),
                               dt=float(z["dt"]), nsteps=int(z["nsteps"]), checkpoint_timesteps=False)
    for k in ("u", "theta"):
        assert torch.equal(again[k], grads[k]), k
    # nested recomputation (the configuration's gradient_checkpointing): each dynamics
    # substep recomputed from its step's checkpoint with only its own tape, sqrt(nsteps)
    # step checkpoints: the same gradients bit for bit
    state = {k: torch.as_tensor(v) for k, v in st0.items()}
    nested = run_simulation.vjp(state, mesh, objective, track_keys=("u", "theta"),
                                config=dict(config(case), gradient_checkpointing=True), dt=float(z["dt"]),
                                nsteps=int(z["nsteps"]))
    for k in ("u", "theta"):
        assert torch.equal(nested[k], grads[k]), k


@pytest.mark.parametrize("case", AD_CASES + AD_OPTION_CASES + AD_TERRAIN_CASES)
def test_mixed_form_gradient_within_1e4_of_reference(case):
    """The mixed form's gradient (float32 stencils in the forward and its taped recompute,
    the reverse pass in float64 about that trajectory) against the reference's float64 VJP:
    rel L2 <= 1e-4."""
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import run_simulation
    z = _npz(case)
    mesh, st0 = mesh_and_state(case)
    nc = int(mesh["nCells"])
    objective = _reference_objective(mesh, z["sp_ref"], nc)
    state = {k: torch.as_tensor(v) for k, v in st0.items()}
    grads = run_simulation.vjp(state, mesh, objective, track_keys=("u", "theta"),
                               config=dict(config(case), config_precision="mixed"), dt=float(z["dt"]),
                               nsteps=int(z["nsteps"]))
    for k in ("u", "theta"):
        a = to_np(grads[k])[:-1]
        b = z[f"grad_{k}"][:-1]
        err = np.linalg.norm(a - b) / np.linalg.norm(b)
        print(f"{case} mixed grad_{k}: rel L2 vs reference {err:.3e}")
        assert err <= 1e-4, (case, k, err)


@pytest.mark.parametrize("case", ("g2_ad", "g2_ad_terrain_fixed"))
def test_differentiable_run_backward_is_the_hand_written_vjp(case):
    """run_simulation(differentiable=True) with the loaded u and theta requiring grad, then
    loss.backward() on the surface-pressure functional of its result: the gradients equal
    run_simulation.vjp's bit for bit (the same reverse pass, run by autograd), with per-step
    checkpoints and with every step's tape kept; a loss through an output whose derivative
    is not built (the scalars) is refused at backward."""
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import run_simulation
    from mpas_dycore_pytorch_gb300.errors import MpasUnsupportedCapabilityError
    z = _npz(case)
    mesh, st0 = mesh_and_state(case)
    nc = int(mesh["nCells"])
    objective = _reference_objective(mesh, z["sp_ref"], nc)
    kw = dict(config=config(case), dt=float(z["dt"]), nsteps=int(z["nsteps"]))
    state = {k: torch.as_tensor(v) for k, v in st0.items()}
    want = run_simulation.vjp(state, mesh, objective, track_keys=("u", "theta"), **kw)
    for tape_all in (False, True):
        state = {k: torch.as_tensor(v) for k, v in st0.items()}
        state["u"] = state["u"].clone().requires_grad_(True)
        state["theta"] = state["theta"].clone().requires_grad_(True)
        out = run_simulation(state, mesh, differentiable=True, checkpoint_timesteps=not tape_all, **kw)
        assert out["rho_zz"].requires_grad and out["u"].requires_grad
        # the tape-all forward advances the dynamics only: no stale scalars in its result
        assert ("scalars" in out) != tape_all
        objective(out).backward()
        for k in ("u", "theta"):
            g = state[k].grad
            assert g is not None and g.device == state[k].device, k
            assert torch.equal(g, want[k].to(g.device)), (k, tape_all)
            err = np.linalg.norm(to_np(g)[:-1] - z[f"grad_{k}"][:-1]) / np.linalg.norm(z[f"grad_{k}"][:-1])
            print(f"{case} tape_all={tape_all} differentiable-run grad_{k}: rel L2 vs reference {err:.3e}")
    # control: the derivative through the scalars is not built, so a loss that reads them is
    # refused rather than differentiated as if they were constant
    state = {k: torch.as_tensor(v) for k, v in st0.items()}
    state["u"] = state["u"].clone().requires_grad_(True)
    out = run_simulation(state, mesh, differentiable=True, **kw)
    with pytest.raises(MpasUnsupportedCapabilityError, match="scalars"):
        (objective(out) + out["scalars"].sum()).backward()
