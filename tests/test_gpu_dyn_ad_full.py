"""The dynamics derivatives against the reference's own at the differentiation workload's
stated size (tests/golden/make_golden_dyn_ad_full.py: level-5 mesh 10242 cells x 41 levels,
16-bit wind, 0.1 m/s sinusoidal w, dt 900 s, 24 steps):

* run_simulation.vjp of the area-weighted squared surface-pressure anomaly with respect to
  the initial u and theta, within the stated 1e-10 relative L2 on the fixture's sampled
  rows and by full-field norm, and the functional itself within 1e-12;
* the mixed form's gradient within the stated 1e-4 of the reference's;
* run_simulation.jvp along the recorded direction, within 1e-10 or, where larger, the
  tangent's own conditioning (its change when u and theta move by one unit in the last
  place; the Smagorinsky coefficient's derivative follows roundoff, see test_gpu_dyn_jvp).

The run starts from the reference run's very inputs (the generated case's digests are
checked first)."""

import json

import numpy as np
import pytest
import torch

from full_size import GOLDEN, case_digest_mismatches
from gpu_helpers import need_gpu, to_np

pytestmark = pytest.mark.gpu

TRACK = ("u", "theta")
JVP_KEYS = ("rho_zz", "pressure_p", "u", "theta_m", "w")


def _fixture():
    path = GOLDEN / "dyn_ad_c2.json"
    if not path.exists():
        pytest.skip("fixture not generated")
    meta = json.loads(path.read_text())
    return meta, dict(np.load(GOLDEN / "dyn_ad_c2.npz"))


def _case(meta):
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.loader import load_case
    bad = case_digest_mismatches(meta)
    assert not bad, f"the generated case differs from the reference run's input: {bad[:5]}"
    cfg = dict(meta["config"])
    st, _ = load_case(CaseSpec(**meta["spec"]), cfg, as_torch=False)
    return st, cfg


def _objective(st, sp_ref):
    from mpas_dycore_pytorch_gb300.diagnostics import physics_interface_surface_pressure, surface_pressure_functional
    dev = torch.device("cuda")
    nc = int(st["nCells"])
    zz = torch.as_tensor(np.asarray(st["zz"]), dtype=torch.float64, device=dev)
    zgrid = torch.as_tensor(np.asarray(st["zgrid"]), dtype=torch.float64, device=dev)
    area = torch.as_tensor(np.asarray(st["areaCell"]), dtype=torch.float64, device=dev)
    ref = torch.as_tensor(sp_ref, dtype=torch.float64, device=dev)

    def objective(out):
        rz = out["rho_zz"]
        sp = physics_interface_surface_pressure(nCells=nc, rho_zz=rz, zz=zz, qv=torch.zeros_like(rz),
                                                pressure_p=out["pressure_p"],
                                                pressure_base=out["pressure_base"].to(dev), zgrid=zgrid)
        return surface_pressure_functional(sp, ref, area, nc)

    return objective


def _compare(meta, arr, tag, got):
    rows = arr[f"{tag}/rows"]
    ref = arr[f"{tag}/values"]
    a = np.asarray(got, dtype=np.float64)
    err = np.linalg.norm(a[rows] - ref) / np.linalg.norm(ref)
    n = a.shape[0] - 1
    norm_ref = np.sqrt(meta[tag]["sumsq"])
    nerr = abs(np.linalg.norm(a[:n]) - norm_ref) / norm_ref
    return max(err, nerr)


def test_gradient_matches_reference_at_workload_size():
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import run_simulation
    meta, arr = _fixture()
    st, cfg = _case(meta)
    state = {k: torch.as_tensor(v) for k, v in st.items() if isinstance(v, np.ndarray)}
    objective = _objective(st, arr["sp_ref"])
    grads = run_simulation.vjp(state, st, objective, track_keys=TRACK, config=cfg, dt=float(meta["dt"]),
                               nsteps=int(meta["nsteps"]))
    for k in TRACK:
        err = _compare(meta, arr, f"grad_{k}", to_np(grads[k]))
        print(f"grad_{k}: rel L2 vs reference {err:.3e}")
        assert err <= 1e-10, (k, err)
    final = run_simulation(state, st, cfg, float(meta["dt"]), nsteps=int(meta["nsteps"]))
    J = float(objective(final))
    print(f"J: {J:.15e} vs reference {meta['J']:.15e}")
    assert abs(J - meta["J"]) <= 1e-12 * abs(meta["J"])


def test_mixed_form_gradient_within_1e4_of_reference_at_workload_size():
    """The mixed form's gradient (float32 stencils in the forward and its taped recompute,
    the reverse pass in float64 about that trajectory) against the reference's float64 VJP:
    rel L2 <= 1e-4."""
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import run_simulation
    meta, arr = _fixture()
    st, cfg = _case(meta)
    state = {k: torch.as_tensor(v) for k, v in st.items() if isinstance(v, np.ndarray)}
    grads = run_simulation.vjp(state, st, _objective(st, arr["sp_ref"]), track_keys=TRACK,
                               config=dict(cfg, config_precision="mixed"), dt=float(meta["dt"]),
                               nsteps=int(meta["nsteps"]))
    for k in TRACK:
        err = _compare(meta, arr, f"grad_{k}", to_np(grads[k]))
        print(f"mixed grad_{k}: rel L2 vs reference {err:.3e}")
        assert err <= 1e-4, (k, err)


def test_tangent_matches_reference_at_workload_size():
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import run_simulation
    from mpas_dycore_pytorch_gb300.cases import _normal
    meta, arr = _fixture()
    st, cfg = _case(meta)
    rng = np.random.default_rng(int(meta["direction_seed"]))
    pert = {}
    for k in TRACK:
        d = _normal(rng, tuple(np.asarray(st[k]).shape)) * (1.0 if k == "u" else 0.1)
        d[-1] = 0.0
        pert[k] = torch.as_tensor(d)
    state = {k: torch.as_tensor(v) for k, v in st.items() if isinstance(v, np.ndarray)}
    kw = dict(config=cfg, dt=float(meta["dt"]), nsteps=int(meta["nsteps"]))
    tan = run_simulation.jvp(state, st, pert, **kw)
    noise = np.random.default_rng(5)
    noisy = dict(state)
    for k in TRACK:
        x = state[k].numpy().copy()
        x[:-1] *= 1.0 + 2.0 ** -52 * noise.choice([-1.0, 0.0, 1.0], size=x[:-1].shape)
        noisy[k] = torch.as_tensor(x)
    tan_n = run_simulation.jvp(noisy, st, pert, **kw)
    fails = []
    for k in JVP_KEYS:
        a = to_np(tan[k])
        err = _compare(meta, arr, f"jvp_{k}", a)
        floor = np.linalg.norm(to_np(tan_n[k])[:-1] - a[:-1]) / np.linalg.norm(a[:-1])
        print(f"jvp_{k}: rel L2 vs reference {err:.3e} (1-ulp input conditioning {floor:.3e})")
        if err > max(1e-10, floor):
            fails.append((k, err, floor))
    assert not fails, fails
