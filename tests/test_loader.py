"""The package loader reproduces the reference loader's runtime dictionaries (golden)."""

import numpy as np
import pytest

from fixtures import CASES, group, load_case


@pytest.mark.parametrize("case", CASES)
def test_loader_matches_reference_loader(case):
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.loader import load_case as pkg_load
    meta, st, _ = load_case(case)
    ref = group(st, "loaded")
    mine, _ = pkg_load(CaseSpec(**meta["spec"]), meta["config"], as_torch=False)
    for k, r in ref.items():
        assert k in mine, k
        g = np.asarray(mine[k])
        assert g.shape == r.shape, (k, g.shape, r.shape)
        if r.dtype.kind in "iu":
            assert np.array_equal(g.astype(np.int64), r.astype(np.int64)), k
        elif r.size:
            scale = max(np.abs(r).max(), 1e-300)
            assert np.abs(g - r).max() <= 1e-14 * scale, k


def test_mesh_generator_properties():
    from mpas_dycore_pytorch_gb300.cases import build_mesh
    m = build_mesh(3)
    nc, ne, nv = m["nCells"], m["nEdges"], m["nVertices"]
    assert (nc, ne, nv) == (642, 1920, 1280)
    R = 6371229.0
    assert abs(m["areaCell"].sum() / (4 * np.pi * R * R) - 1) < 1e-12
    assert np.allclose(m["kiteAreasOnVertex"].sum(1), m["areaTriangle"], rtol=1e-12)
    # TRiSK weights are antisymmetric (energy-conserving Coriolis term)
    eoe, w = m["edgesOnEdge"] - 1, m["weightsOnEdge"]
    dc, dv = m["dcEdge"], m["dvEdge"]
    W = {}
    for e in range(ne):
        for j in range(m["nEdgesOnEdge"][e]):
            W[(e, eoe[e, j])] = w[e, j] * dc[e] / dv[eoe[e, j]]
    assert max(abs(W[(a, b)] + W[(b, a)]) for (a, b) in W) < 1e-14
