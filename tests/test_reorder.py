"""Mesh reordering: the RCM order against the reference's own output (golden), the
space-filling-curve order (a valid permutation, consistent connectivity, exact round
trip), and (GPU) a step on the reordered mesh equal bit for bit to the original step."""

import pathlib

import numpy as np
import pytest
import torch

from fixtures import group, load_case
from gpu_helpers import need_gpu

GOLD = np.load(pathlib.Path(__file__).resolve().parent / "golden" / "rcm_g2.npz")


@pytest.fixture(scope="module")
def g2():
    meta, st, _ = load_case("g2_explicit")
    return dict(group(st, "loaded"))


def test_rcm_matches_reference(g2):
    from mpas_dycore_pytorch_gb300.build import build
    from mpas_dycore_pytorch_gb300.reorder import apply_rcm_reordering
    build()
    state = {k: g2[k] for k in ("u", "theta", "rho", "w", "scalars")}
    rst, rmesh = apply_rcm_reordering(state, g2)
    for k, v in rmesh["_rcm_permutation"].items():
        assert np.array_equal(v.numpy(), GOLD[f"perm/{k}"]), k
    for key in [k for k in GOLD.files if k.startswith("mesh/")]:
        assert np.array_equal(np.asarray(rmesh[key[5:]]), GOLD[key]), key
    for key in [k for k in GOLD.files if k.startswith("state/")]:
        assert np.array_equal(np.asarray(rst[key[6:]]), GOLD[key]), key


def _check_consistent(m):
    nc, ne = int(np.asarray(m["nCells"])), int(np.asarray(m["nEdges"]))
    coe, eoc, neoc = np.asarray(m["cellsOnEdge"]), np.asarray(m["edgesOnCell"]), np.asarray(m["nEdgesOnCell"])
    for c in range(nc):
        for j in range(neoc[c]):
            e = eoc[c, j] - 1
            assert c + 1 in coe[e], (c, e)


def test_sfc_is_a_permutation_with_consistent_connectivity_and_exact_round_trip(g2):
    from mpas_dycore_pytorch_gb300.build import build
    from mpas_dycore_pytorch_gb300.reorder import apply_sfc_reordering, restore_order
    build()
    state = {k: g2[k] for k in ("u", "theta", "w")}
    rst, rmesh, perm = apply_sfc_reordering(state, g2)
    nc, ne, nv = (int(np.asarray(g2[k])) for k in ("nCells", "nEdges", "nVertices"))
    for p, n in ((perm.cell_new_to_old, nc), (perm.edge_new_to_old, ne), (perm.vertex_new_to_old, nv)):
        assert np.array_equal(np.sort(p), np.arange(n))
    assert not np.array_equal(perm.cell_new_to_old, np.arange(nc))  # it does reorder
    _check_consistent(rmesh)
    back = restore_order(rmesh, perm, (nc, ne, nv))
    for k, v in g2.items():
        if np.ndim(v) > 0:
            assert np.array_equal(np.asarray(back[k]), np.asarray(v)), k
    sback = restore_order(rst, perm, (nc, ne, nv))
    for k in state:
        assert np.array_equal(sback[k], state[k])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ("float64", "mixed"))
def test_step_on_reordered_mesh_is_bit_identical(precision):
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import Model
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.device import STATE_KEYS
    from mpas_dycore_pytorch_gb300.loader import load_case as synth
    from mpas_dycore_pytorch_gb300.reorder import apply_sfc_reordering, restore_order
    cfg = {"config_time_integration_order": 3, "config_len_disp": 120000.0, "config_monotonic": True,
           "config_dt": 600.0}
    st, _ = synth(CaseSpec(level=4, nlev=20, seed=5, n_bumps=4, n_tracers=2), cfg, as_torch=False)
    dims = tuple(int(np.asarray(st[k])) for k in ("nCells", "nEdges", "nVertices"))
    outs = []
    for reorder in (False, True):
        s = st
        if reorder:
            s, _, perm = apply_sfc_reordering(st, st)
        m = Model(s, cfg, 600.0, num_scalars=2, precision=precision)
        m.prepare(s)
        for _ in range(2):
            m.step()
        res = {k: m.state.f[k] for k in STATE_KEYS}
        if reorder:
            res = restore_order(res, perm, dims)
        outs.append(res)
    for k in STATE_KEYS:
        assert torch.equal(outs[0][k][:-1], outs[1][k][:-1]), (precision, k)


@pytest.mark.gpu
def test_reference_rcm_option_returns_results_in_rcm_order():
    need_gpu()
    import mpas_dycore_pytorch_gb300 as gb
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.loader import load_case as synth
    from mpas_dycore_pytorch_gb300.reorder import apply_permutation, compute_rcm_permutation
    cfg = {"config_time_integration_order": 3, "config_len_disp": 120000.0, "config_monotonic": False,
           "config_dt": 600.0}
    st, _ = synth(CaseSpec(level=3, nlev=12, seed=6, n_bumps=2, n_tracers=1), cfg, as_torch=False)
    dims = tuple(int(np.asarray(st[k])) for k in ("nCells", "nEdges", "nVertices"))
    perm = compute_rcm_permutation(st)
    plain = gb.run_simulation(dict(st), dict(st), cfg, 600.0, 1, "cuda")
    mesh = dict(st)
    rcm = gb.run_simulation(dict(st), mesh, dict(cfg, config_mesh_reordering_rcm=True), 600.0, 1, "cuda")
    assert mesh.get("_rcm_applied") is True  # the caller's mesh is updated, as in the reference
    want = apply_permutation({k: plain[k] for k in ("u", "w", "theta_m", "rho_zz")}, perm, dims)
    for k, v in want.items():
        assert torch.equal(rcm[k][:-1], v[:-1]), k


@pytest.mark.gpu
def test_model_sfc_order_is_transparent():
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import Model
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.device import STATE_KEYS
    from mpas_dycore_pytorch_gb300.loader import load_case as synth
    cfg = {"config_time_integration_order": 3, "config_len_disp": 120000.0, "config_monotonic": True,
           "config_dt": 600.0}
    st, _ = synth(CaseSpec(level=3, nlev=14, seed=8, n_bumps=3, n_tracers=2), cfg, as_torch=False)
    native = Model(st, cfg, 600.0, num_scalars=2)
    sfc = Model(st, cfg, 600.0, num_scalars=2, order="sfc")
    native.prepare(st)
    sfc.prepare(st)
    native.step()
    sfc.step()
    a, b = native.export(), sfc.export()
    for k in STATE_KEYS:
        assert torch.equal(a[k][:-1], b[k][:-1]), k
    # a boundary in the caller's order continues identically in both
    host = {k: a[k].cpu() for k in STATE_KEYS}
    native.load_boundary(host)
    sfc.load_boundary(host)
    native.step()
    sfc.step()
    a, b = native.export(), sfc.export()
    for k in STATE_KEYS:
        assert torch.equal(a[k][:-1], b[k][:-1]), k


@pytest.mark.gpu
@pytest.mark.parametrize("order", ["native", "sfc"])
def test_host_chain_through_export_to_matches_resident_steps(order):
    """Steps chained through pinned host buffers (load_boundary -> step -> export_to,
    the copies out overlapping the next copies in) equal the same steps kept on the
    device, bit for bit; the padding rows come back too."""
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import Model
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.device import STATE_KEYS
    from mpas_dycore_pytorch_gb300.loader import load_case as synth
    cfg = {"config_time_integration_order": 3, "config_len_disp": 120000.0, "config_monotonic": True,
           "config_dt": 600.0}
    st, _ = synth(CaseSpec(level=3, nlev=14, seed=9, n_bumps=3, n_tracers=2), cfg, as_torch=False)
    resident = Model(st, cfg, 600.0, num_scalars=2, order=order)
    chained = Model(st, cfg, 600.0, num_scalars=2, order=order)
    resident.prepare(st)
    chained.prepare(st)
    start = resident.export()
    host = {k: torch.empty(start[k].shape, dtype=torch.float64, pin_memory=True) for k in STATE_KEYS}
    for k in STATE_KEYS:
        host[k].copy_(start[k])
    for _ in range(3):
        resident.step()
        chained.load_boundary(host)
        chained.step()
        chained.export_to(host)
    chained.wait_exports()
    torch.cuda.synchronize()
    want = resident.export()
    for k in STATE_KEYS:
        assert torch.equal(host[k], want[k].cpu()), k
    with pytest.raises(Exception):
        chained.export_to({"not_a_field": host["u"]})


@pytest.mark.gpu
@pytest.mark.parametrize("order,coupled", [("native", False), ("sfc", False), ("sfc", True)])
def test_step_host_in_two_parts_matches_resident_steps(order, coupled):
    """Model.step_host (the step's two parts as graphs, the final fields copied out while
    the transport runs) equals whole steps kept on the device, bit for bit."""
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import Model
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.device import STATE_KEYS
    from mpas_dycore_pytorch_gb300.loader import load_case as synth
    cfg = {"config_time_integration_order": 3, "config_len_disp": 120000.0, "config_monotonic": True,
           "config_dt": 600.0, "config_split_dynamics_transport": not coupled}
    st, _ = synth(CaseSpec(level=3, nlev=14, seed=5, n_bumps=3, n_tracers=2), cfg, as_torch=False)
    resident = Model(st, cfg, 600.0, num_scalars=2, order=order)
    hosted = Model(st, cfg, 600.0, num_scalars=2, order=order)
    resident.prepare(st)
    hosted.prepare(st)
    start = resident.export()
    host = {k: torch.empty(start[k].shape, dtype=torch.float64, pin_memory=True) for k in STATE_KEYS}
    for k in STATE_KEYS:
        host[k].copy_(start[k])
    hosted.step_host(host)  # eager parts
    resident.step()
    hosted.capture_graph_parts()
    for _ in range(2):  # graph-replayed parts
        hosted.step_host(host)
        resident.step()
    hosted.wait_exports()
    torch.cuda.synchronize()
    want = resident.export()
    for k in STATE_KEYS:
        assert torch.equal(host[k], want[k].cpu()), k


@pytest.mark.gpu
@pytest.mark.parametrize("order", ["native", "sfc"])
def test_run_host_pipeline_matches_resident_steps(order):
    """Model.run_host (every step's boundary copied in from and out to pinned host
    tensors, the copies pipelined with the steps on two copy streams) equals the same
    steps kept on the device, bit for bit."""
    need_gpu()
    from mpas_dycore_pytorch_gb300.api import Model
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.device import STATE_KEYS
    from mpas_dycore_pytorch_gb300.loader import load_case as synth
    cfg = {"config_time_integration_order": 3, "config_len_disp": 120000.0, "config_monotonic": True,
           "config_dt": 600.0}
    st, _ = synth(CaseSpec(level=3, nlev=14, seed=6, n_bumps=3, n_tracers=2), cfg, as_torch=False)
    resident = Model(st, cfg, 600.0, num_scalars=2, order=order)
    hosted = Model(st, cfg, 600.0, num_scalars=2, order=order)
    resident.prepare(st)
    hosted.prepare(st)
    start = resident.export()
    host = {k: torch.empty(start[k].shape, dtype=torch.float64, pin_memory=True) for k in STATE_KEYS}
    for k in STATE_KEYS:
        host[k].copy_(start[k])
    hosted.run_host(host, 1)
    hosted.run_host(host, 3)
    for _ in range(4):
        resident.step()
    torch.cuda.synchronize()
    want = resident.export()
    for k in STATE_KEYS:
        assert torch.equal(host[k], want[k].cpu()), k
