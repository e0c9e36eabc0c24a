"""Ensemble union layout (CPU): counts, connectivity remapping and member split."""

import numpy as np
import pytest
import torch

from mpas_dycore_pytorch_gb300.cases import CaseSpec
from mpas_dycore_pytorch_gb300.ensemble import CONNECTIVITY, member_cases, split_member, stack_members
from mpas_dycore_pytorch_gb300.errors import MpasConfigError
from mpas_dycore_pytorch_gb300.loader import load_case


@pytest.fixture(scope="module")
def members():
    a = member_cases(CaseSpec(level=2, nlev=12, n_bumps=2, n_tracers=2), seeds=[0, 1])
    b, _ = load_case(CaseSpec(level=3, nlev=12, seed=2, n_bumps=2, n_tracers=2), None, as_torch=False)
    return a + [b]


def test_union_counts_and_connectivity(members):
    union, layouts = stack_members(members)
    n = {k: [int(np.asarray(m[k])) for m in members] for k in ("nCells", "nEdges", "nVertices")}
    assert union["nCells"] == sum(n["nCells"]) and union["nEdges"] == sum(n["nEdges"])
    tot = {"cell": union["nCells"], "edge": union["nEdges"], "vertex": union["nVertices"]}
    rows = {"cellsOnCell": "cell", "cellsOnEdge": "edge", "edgesOnCell": "cell", "edgesOnEdge": "edge",
            "verticesOnEdge": "edge", "advCellsForEdge": "edge", "edgesOnVertex": "vertex"}
    for key, row_kind in rows.items():
        tgt = CONNECTIVITY[key]
        u = np.asarray(union[key])
        for b, (m, lay) in enumerate(zip(members, layouts)):
            lo, hi = {"cell": lay.cells, "edge": lay.edges, "vertex": lay.vertices}[row_kind]
            mine = np.asarray(m[key])[:hi - lo]
            got = u[lo:hi, :mine.shape[1]]
            nt = {"cell": lay.cells, "edge": lay.edges, "vertex": lay.vertices}[tgt]
            inside = (mine >= 1) & (mine <= nt[1] - nt[0])
            assert np.array_equal(got[inside], mine[inside] + nt[0]), (key, b)
            assert np.all((got[~inside] == 0) | (got[~inside] == tot[tgt] + 1)), (key, b)
            assert np.all(got[inside] >= nt[0] + 1) and np.all(got[inside] <= nt[1])  # never crosses members
    assert np.asarray(union["theta"]).shape[0] == tot["cell"] + 1


def test_split_member_round_trip(members):
    union, layouts = stack_members(members)
    dims = {"cell": union["nCells"], "edge": union["nEdges"], "vertex": union["nVertices"]}
    t = {"theta": torch.as_tensor(np.asarray(union["theta"])), "u": torch.as_tensor(np.asarray(union["u"]))}
    for m, lay in zip(members, layouts):
        part = split_member(t, lay, dims)
        assert torch.equal(part["theta"][:-1], torch.as_tensor(np.asarray(m["theta"]))[:-1])
        assert torch.equal(part["u"][:-1], torch.as_tensor(np.asarray(m["u"]))[:-1])


def test_members_must_share_vertical_grid(members):
    other, _ = load_case(CaseSpec(level=2, nlev=14, seed=3, n_bumps=1, n_tracers=2), None, as_torch=False)
    with pytest.raises(MpasConfigError):
        stack_members([members[0], other])
