"""Mesh reordering: the reference's RCM order and the space-filling-curve order.

``apply_rcm_reordering`` restates the reference's utility (mpas_pytorch/
mesh_reordering.py:243): reverse Cuthill-McKee (scipy's ``reverse_cuthill_mckee``, as the
reference calls it) of the cell graph (cellsOnCell) and of the vertex graph (through
verticesOnEdge), edges sorted by (min, max) new cell id then old index; rows of every
cell / edge / vertex array are permuted (the padding row stays last) and connectivity
values remapped.  ``apply_sfc_reordering`` is the same operation with the cell and vertex
orders taken along a 3-D Hilbert curve (``mpasg_sfc_order``, host C++) and the same edge
rule (``mpasg_edge_order``); ``restore_order`` maps results back.  Relabelling keeps every
entity's connectivity slot order, so a step on a reordered mesh is bit-identical to the
step on the original mesh after the inverse permutation.
"""

from __future__ import annotations

import ctypes as C
import dataclasses
from typing import Any, Mapping

import numpy as np
import torch

from . import _lib

CELL_INDEX_KEYS = {"cellsOnEdge", "cellsOnCell", "cellsOnVertex", "advCellsForEdge"}
EDGE_INDEX_KEYS = {"edgesOnCell", "edgesOnEdge", "edgesOnVertex"}
VERTEX_INDEX_KEYS = {"verticesOnEdge", "verticesOnCell"}


@dataclasses.dataclass(frozen=True)
class Permutation:
    """new_to_old / old_to_new index maps (0-based int64) for cells, edges, vertices."""

    cell_new_to_old: np.ndarray
    edge_new_to_old: np.ndarray
    vertex_new_to_old: np.ndarray

    @property
    def cell_old_to_new(self) -> np.ndarray:
        return _inverse(self.cell_new_to_old)

    @property
    def edge_old_to_new(self) -> np.ndarray:
        return _inverse(self.edge_new_to_old)

    @property
    def vertex_old_to_new(self) -> np.ndarray:
        return _inverse(self.vertex_new_to_old)

    def inverse(self) -> "Permutation":
        return Permutation(self.cell_old_to_new, self.edge_old_to_new, self.vertex_old_to_new)


def _np(x) -> np.ndarray:
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy()
    return np.asarray(x)


def _int(x) -> int:
    return int(_np(x).reshape(-1)[0])


def _inverse(new_to_old: np.ndarray) -> np.ndarray:
    inv = np.empty_like(new_to_old)
    inv[new_to_old] = np.arange(new_to_old.size, dtype=new_to_old.dtype)
    return inv


def _dims(mesh: Mapping[str, Any]) -> tuple[int, int, int]:
    return _int(mesh["nCells"]), _int(mesh["nEdges"]), _int(mesh["nVertices"])


def _edge_order(mesh, nc: int, ne: int, cell_old_to_new: np.ndarray) -> np.ndarray:
    lib = _lib.load()
    coe = np.ascontiguousarray(_np(mesh["cellsOnEdge"])[:ne, :2], dtype=np.int64)
    c2n = np.ascontiguousarray(cell_old_to_new, dtype=np.int64)
    out = np.empty(ne, dtype=np.int64)
    rc = lib.mpasg_edge_order(ne, nc, coe.ctypes.data_as(C.c_void_p), c2n.ctypes.data_as(C.c_void_p),
                              out.ctypes.data_as(C.c_void_p))
    _lib.check(rc, "mpasg_edge_order")
    return out


def compute_sfc_permutation(mesh: Mapping[str, Any]) -> Permutation:
    """Hilbert-curve order of cells and vertices (their x/y/z centres) and the edge rule."""
    lib = _lib.load()
    nc, ne, nv = _dims(mesh)

    def curve(prefix: str, n: int) -> np.ndarray:
        xyz = [np.ascontiguousarray(_np(mesh[a + prefix])[:n], dtype=np.float64) for a in ("x", "y", "z")]
        out = np.empty(n, dtype=np.int64)
        rc = lib.mpasg_sfc_order(n, *(a.ctypes.data_as(C.c_void_p) for a in xyz), out.ctypes.data_as(C.c_void_p))
        _lib.check(rc, "mpasg_sfc_order")
        return out

    cells = curve("Cell", nc)
    verts = curve("Vertex", nv)
    edges = _edge_order(mesh, nc, ne, _inverse(cells))
    return Permutation(cells, edges, verts)


def compute_rcm_permutation(mesh: Mapping[str, Any]) -> Permutation:
    """The reference's orders (mesh_reordering.py:44-103): RCM of the cell graph and of the
    vertex graph, edges by (min, max) new cell id then old index."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import reverse_cuthill_mckee

    nc, ne, nv = _dims(mesh)

    def rcm(n, rows, cols):
        if n <= 0:
            return np.arange(0, dtype=np.int64)
        if rows.size == 0:
            return np.arange(n, dtype=np.int64)
        g = coo_matrix((np.ones(rows.shape[0], dtype=np.int8), (rows, cols)), shape=(n, n)).tocsr()
        g = (g + g.T).tocsr()
        g.data[:] = 1
        return reverse_cuthill_mckee(g, symmetric_mode=True).astype(np.int64)

    coc = _np(mesh["cellsOnCell"])[:nc].astype(np.int64)
    rows = np.repeat(np.arange(nc, dtype=np.int64), coc.shape[1])
    cols = coc.reshape(-1) - 1
    ok = (cols >= 0) & (cols < nc)
    cells = rcm(nc, rows[ok], cols[ok])
    voe = _np(mesh["verticesOnEdge"])[:ne, :2].astype(np.int64) - 1
    ok = (voe[:, 0] >= 0) & (voe[:, 0] < nv) & (voe[:, 1] >= 0) & (voe[:, 1] < nv)
    verts = rcm(nv, np.concatenate([voe[ok, 0], voe[ok, 1]]), np.concatenate([voe[ok, 1], voe[ok, 0]]))
    edges = _edge_order(mesh, nc, ne, _inverse(cells))
    return Permutation(cells, edges, verts)


def _take_rows(value, perm: np.ndarray):
    n = perm.size
    if isinstance(value, torch.Tensor):
        p = torch.as_tensor(perm, device=value.device)
        head = value[:n][p]
        return head if value.shape[0] == n else torch.cat([head, value[n:n + 1]], 0)
    a = np.asarray(value)
    head = a[:n][perm]
    return head if a.shape[0] == n else np.concatenate([head, a[n:n + 1]], 0)


def _remap_values(value, old_to_new: np.ndarray, n: int):
    if isinstance(value, torch.Tensor):
        out = value.clone()
        ok = (out >= 1) & (out <= n)
        m = torch.as_tensor(old_to_new, device=value.device)
        out[ok] = (m[(out[ok] - 1).long()] + 1).to(out.dtype)
        return out
    a = np.array(value, copy=True)
    ok = (a >= 1) & (a <= n)
    a[ok] = (old_to_new[a[ok].astype(np.int64) - 1] + 1).astype(a.dtype)
    return a


def apply_permutation(data: Mapping[str, Any], perm: Permutation, dims: tuple[int, int, int]) -> dict:
    """Rows of every cell / edge / vertex array (N or N+1 rows) permuted new <- old and
    connectivity values remapped old -> new (1-based, sentinels kept)."""
    nc, ne, nv = dims
    c2n, e2n, v2n = perm.cell_old_to_new, perm.edge_old_to_new, perm.vertex_old_to_new
    out: dict[str, Any] = {}
    for key, value in data.items():
        if isinstance(value, (np.ndarray, torch.Tensor)) and np.ndim(value) > 0:
            n0 = value.shape[0]
            if n0 in (nc, nc + 1):
                value = _take_rows(value, perm.cell_new_to_old)
            elif n0 in (ne, ne + 1):
                value = _take_rows(value, perm.edge_new_to_old)
            elif n0 in (nv, nv + 1):
                value = _take_rows(value, perm.vertex_new_to_old)
            kind = value.dtype.kind if isinstance(value, np.ndarray) else ("i" if not value.is_floating_point() else "f")
            if kind in "iu":
                if key in CELL_INDEX_KEYS:
                    value = _remap_values(value, c2n, nc)
                elif key in EDGE_INDEX_KEYS:
                    value = _remap_values(value, e2n, ne)
                elif key in VERTEX_INDEX_KEYS:
                    value = _remap_values(value, v2n, nv)
        out[key] = value
    return out


def restore_order(data: Mapping[str, Any], perm: Permutation, dims: tuple[int, int, int]) -> dict:
    """Inverse of ``apply_permutation`` (results of a reordered run in the original order)."""
    return apply_permutation(data, perm.inverse(), dims)


def _perm_record(perm: Permutation) -> dict:
    t = lambda a: torch.as_tensor(a)
    return {"cell_new_to_old": t(perm.cell_new_to_old), "edge_new_to_old": t(perm.edge_new_to_old),
            "vertex_new_to_old": t(perm.vertex_new_to_old), "cell_old_to_new": t(perm.cell_old_to_new),
            "edge_old_to_new": t(perm.edge_old_to_new), "vertex_old_to_new": t(perm.vertex_old_to_new)}


def apply_rcm_reordering(state: Mapping[str, Any], mesh: Mapping[str, Any]) -> tuple[dict, dict]:
    """Reordered copies of ``state`` and ``mesh`` in the reference's RCM order; the mesh
    carries ``_rcm_applied`` and ``_rcm_permutation`` as in the reference."""
    dims = _dims(mesh)
    perm = compute_rcm_permutation(mesh)
    st, me = apply_permutation(state, perm, dims), apply_permutation(mesh, perm, dims)
    me["_rcm_applied"] = True
    me["_rcm_permutation"] = _perm_record(perm)
    return st, me


def apply_sfc_reordering(state: Mapping[str, Any], mesh: Mapping[str, Any]) -> tuple[dict, dict, Permutation]:
    """Reordered copies of ``state`` and ``mesh`` along the Hilbert curve, and the
    permutation (``restore_order`` maps results back)."""
    dims = _dims(mesh)
    perm = compute_sfc_permutation(mesh)
    st, me = apply_permutation(state, perm, dims), apply_permutation(mesh, perm, dims)
    me["_sfc_applied"] = True
    return st, me, perm
