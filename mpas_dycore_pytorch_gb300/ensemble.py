"""Batched ensembles: B members stepped as one disjoint union of their meshes.

Members may have meshes of different sizes; they share the vertical grid, the number of
scalars and the namelist options (one ``mpasg_config``).  ``stack_members`` concatenates
the members' cells, edges and vertices (the padded reference layout: N+1 rows, 1-based
connectivity with sentinels 0 / N+1) into one union mesh whose connectivity never crosses
members; every kernel's flat (entity, level) index space then covers all members, so
each kernel is one launch over a (member, cell-block) work list and a step is one CUDA
graph for the whole ensemble.  No stage reduces across cells, so every member's result is
bit-identical to running that member alone (tests/test_gpu_ensemble.py).
"""

from __future__ import annotations

import dataclasses
from typing import Any, Mapping, Sequence

import numpy as np
import torch

from .errors import MpasConfigError

# connectivity arrays: the entity their (1-based) values index
CONNECTIVITY = {
    "cellsOnCell": "cell", "cellsOnEdge": "cell", "cellsOnVertex": "cell", "advCellsForEdge": "cell",
    "edgesOnCell": "edge", "edgesOnEdge": "edge", "edgesOnVertex": "edge",
    "verticesOnCell": "vertex", "verticesOnEdge": "vertex",
}
GLOBAL_IDS = {"indexToCellID": "cell", "indexToEdgeID": "edge", "indexToVertexID": "vertex"}
COUNTS = {"nCells": "cell", "nEdges": "edge", "nVertices": "vertex"}
MAXIMA = ("maxEdges", "maxEdges2", "nAdvCellsMax")


def _np(x) -> np.ndarray:
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy()
    return np.asarray(x)


def _int(x) -> int:
    return int(_np(x).reshape(-1)[0])


@dataclasses.dataclass(frozen=True)
class MemberLayout:
    """Row ranges of one member inside the union (0-based, active rows only)."""

    cells: tuple[int, int]
    edges: tuple[int, int]
    vertices: tuple[int, int]


def _kind(shape0: int, n: dict) -> str | None:
    hits = [k for k in ("cell", "edge", "vertex") if shape0 == n[k] + 1]
    if len(hits) > 1:
        raise MpasConfigError(f"ambiguous entity dimension {shape0} (cells/edges/vertices coincide)")
    return hits[0] if hits else None


def stack_members(members: Sequence[Mapping[str, Any]]) -> tuple[dict, list[MemberLayout]]:
    """Union of member dictionaries (reference layout); returns ``(union, layouts)``."""
    if not members:
        raise MpasConfigError("an ensemble needs at least one member")
    for key in ("nVertLevels", "num_scalars"):
        vals = {_int(m[key]) for m in members if key in m}
        if len(vals) > 1:
            raise MpasConfigError(f"ensemble members differ in {key}: {sorted(vals)}; "
                                  "members must share the vertical grid and options")
    dims = [{"cell": _int(m["nCells"]), "edge": _int(m["nEdges"]), "vertex": _int(m["nVertices"])} for m in members]
    total = {k: sum(d[k] for d in dims) for k in ("cell", "edge", "vertex")}
    offs, layouts = [], []
    acc = {"cell": 0, "edge": 0, "vertex": 0}
    for d in dims:
        offs.append(dict(acc))
        layouts.append(MemberLayout(*((acc[k], acc[k] + d[k]) for k in ("cell", "edge", "vertex"))))
        for k in acc:
            acc[k] += d[k]
    first = members[0]
    union: dict[str, Any] = {}
    for key, v0 in first.items():
        a0 = _np(v0)
        if key in COUNTS:
            union[key] = total[COUNTS[key]]
            continue
        if key in MAXIMA:
            union[key] = max(_int(m[key]) for m in members)
            continue
        kind = _kind(a0.shape[0], dims[0]) if a0.ndim >= 1 else None
        if kind is None:  # scalars and per-level arrays: identical across members
            for b, m in enumerate(members[1:], 1):
                if key not in m or not np.array_equal(_np(m[key]), a0):
                    raise MpasConfigError(f"ensemble members differ in {key!r} (member {b}); "
                                          "members must share the vertical grid and options")
            union[key] = v0
            continue
        parts = []
        width = max(_np(m[key]).shape[1] for m in members) if a0.ndim >= 2 else None
        for b, m in enumerate(members):
            a = _np(m[key])
            if _kind(a.shape[0], dims[b]) != kind:
                raise MpasConfigError(f"{key!r} of member {b} has shape {a.shape}")
            a = a[:dims[b][kind]]
            if width is not None and a.shape[1] < width:  # slot arrays of smaller maxima
                pad = np.zeros((a.shape[0], width - a.shape[1]) + a.shape[2:], dtype=a.dtype)
                a = np.concatenate([a, pad], axis=1)
            if key in CONNECTIVITY:
                tgt = CONNECTIVITY[key]
                n_b = dims[b][tgt]
                a = a.astype(np.int64)
                a = np.where((a >= 1) & (a <= n_b), a + offs[b][tgt], np.where(a == 0, 0, total[tgt] + 1))
            elif key in GLOBAL_IDS:
                a = a.astype(np.int64) + offs[b][GLOBAL_IDS[key]]
            parts.append(a)
        pad_row = _np(v0)[dims[0][kind]:dims[0][kind] + 1]
        if width is not None and pad_row.shape[1] < width:
            pad_row = np.concatenate([pad_row, np.zeros((1, width - pad_row.shape[1]) + pad_row.shape[2:],
                                                         dtype=pad_row.dtype)], axis=1)
        if key in CONNECTIVITY:
            pad_row = np.zeros_like(pad_row, dtype=np.int64)
        try:
            out = np.concatenate(parts + [pad_row.astype(parts[0].dtype)], axis=0)
        except ValueError as exc:
            raise MpasConfigError(f"ensemble members disagree in the shape of {key!r}: {exc}") from exc
        if key in CONNECTIVITY or key in GLOBAL_IDS:
            out = out.astype(a0.dtype)
        union[key] = out
    return union, layouts


def split_member(union_state: Mapping[str, Any], layout: MemberLayout, union_dims: Mapping[str, int]) -> dict:
    """Member rows of union-layout arrays (entity arrays get a zero padding row)."""
    out = {}
    rng = {"cell": layout.cells, "edge": layout.edges, "vertex": layout.vertices}
    for key, v in union_state.items():
        if not isinstance(v, torch.Tensor) or v.dim() == 0:
            continue
        kind = _kind(v.shape[0], union_dims)
        if kind is None:
            continue
        lo, hi = rng[kind]
        part = v[lo:hi]
        out[key] = torch.cat([part, torch.zeros_like(part[:1])], 0)
    return out


def member_cases(spec, seeds: Sequence[int], config: Mapping[str, Any] | None = None, u_noise: float = 0.0):
    """Loaded member dictionaries on one mesh: each member's initial state from its seed
    (theta bumps, optional wind noise); the mesh and its derived fields are built once."""
    from .cases import build_mesh, initial_state
    from .loader import _pad, load_case

    base, _ = load_case(dataclasses.replace(spec, seed=int(seeds[0]), u_noise=u_noise), config, as_torch=False)
    mesh = build_mesh(spec.level)
    out = [base]
    for s in seeds[1:]:
        init = initial_state(mesh, dataclasses.replace(spec, seed=int(s), u_noise=u_noise))
        m = dict(base)
        for key in ("u", "w", "theta", "rho", "scalars", "qv"):
            m[key] = _pad(np.asarray(init[key], dtype=np.float64))
        out.append(m)
    return out


class Ensemble:
    """B members stepped together on one GPU (see module docstring)."""

    def __init__(self, members: Sequence[Mapping[str, Any]], config: Mapping[str, Any] | None, dt: float,
                 precision: str | None = None, device: str | torch.device = "cuda", order: str = "native"):
        """``order="sfc"``: each member is put in Hilbert-curve order before stacking (so a
        member's neighbours stay close in memory); ``member_state`` returns the member's
        own order."""
        from .api import Model
        self._perms = None
        if order == "sfc":
            from .reorder import apply_permutation, compute_sfc_permutation
            self._perms = []
            reordered = []
            for m in members:
                dims = tuple(_int(m[k]) for k in ("nCells", "nEdges", "nVertices"))
                perm = compute_sfc_permutation(m)
                self._perms.append((perm, dims))
                reordered.append(apply_permutation(m, perm, dims))
            members = reordered
        elif order != "native":
            raise MpasConfigError(f"order must be 'native' or 'sfc', got {order!r}")
        union, self.layouts = stack_members(members)
        self.union_dims = {"cell": _int(union["nCells"]), "edge": _int(union["nEdges"]),
                           "vertex": _int(union["nVertices"])}
        ns = int(_np(union["scalars"]).shape[-1])
        self.model = Model(union, config, dt, num_scalars=ns, device=device, precision=precision)
        self.model.prepare(union)
        self.cell_levels = self.union_dims["cell"] * self.model.dmesh.nVertLevels

    def step(self) -> None:
        self.model.step()

    def capture_graph(self) -> None:
        self.model.capture_graph()

    def member_state(self, b: int) -> dict:
        out = split_member(self.model.export(), self.layouts[b], self.union_dims)
        if self._perms is not None:
            from .reorder import restore_order
            perm, dims = self._perms[b]
            out = restore_order(out, perm, dims)
        return out


class EnsembleGroups:
    """Members on several vertical grids (or with different timesteps / options), e.g. 96
    members of 10242 cells x 41 levels beside 32 members of 40962 cells x 55 levels.

    The level count is a dimension of every kernel's index space, so members sharing a
    vertical grid and options form one union (``Ensemble``) and the groups step side by
    side: ``capture_graph`` records every group's large step into ONE CUDA graph, each
    group on its own stream forked from and joined back to the capturing stream, so a
    replay launches the whole ensemble at once and the groups' kernels overlap.  Each
    member's result is the same as in its group alone (bit-identical in float64: the
    groups share no memory).
    """

    def __init__(self, groups: Sequence[tuple[Sequence[Mapping[str, Any]], Mapping[str, Any] | None, float]],
                 precision: str | None = None, device: str | torch.device = "cuda", order: str = "native"):
        if not groups:
            raise MpasConfigError("an ensemble needs at least one group")
        self.groups = [Ensemble(members, config, dt, precision=precision, device=device, order=order)
                       for members, config, dt in groups]
        self.cell_levels = sum(g.cell_levels for g in self.groups)
        self._graph = None
        self._streams = None

    def autotune(self) -> list[dict]:
        return [g.model.autotune() for g in self.groups]

    def step(self) -> None:
        if self._graph is not None:
            self._graph.replay()
        else:
            for g in self.groups:
                g.model.step()

    def capture_graph(self) -> None:
        """One graph for all groups (fork / join over one stream per group)."""
        import ctypes as C

        from . import _lib

        torch.cuda.synchronize()
        main = torch.cuda.Stream()
        side = [torch.cuda.Stream() for _ in self.groups]
        main.wait_stream(torch.cuda.current_stream())
        graph = torch.cuda.CUDAGraph()
        rcs = []
        with torch.cuda.stream(main):
            with torch.cuda.graph(graph, stream=main):
                for g, s in zip(self.groups, side):
                    s.wait_stream(main)
                    m = g.model
                    rcs.append(m.lib.mpasg_step(C.byref(m.dmesh.struct), C.byref(m.cstruct),
                                                C.byref(m.state.struct), C.c_void_p(s.cuda_stream)))
                    main.wait_stream(s)
        torch.cuda.current_stream().wait_stream(main)
        for rc in rcs:
            _lib.check(rc, "mpasg_step (ensemble capture)")
        self._graph = graph
        self._streams = (main, side)

    def check_finite(self) -> int:
        return sum(g.model.check_finite() for g in self.groups)

    def member_state(self, group: int, b: int) -> dict:
        return self.groups[group].member_state(b)

    @property
    def state_bytes(self) -> int:
        return sum(g.model.state.bytes for g in self.groups)
