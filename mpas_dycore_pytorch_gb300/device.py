"""Device-resident mesh and state for the CUDA step.

``DeviceMesh`` uploads the reference's static arrays once (1-based padded connectivity is
converted to 0-based int32 whose missing neighbours point at the padding row).
``DeviceState`` owns every field of ``mpasg_fields`` (include/mpasg.h) as float64 device
tensors in the reference layout (rows = entity, levels fastest, one padding row) and
converts to and from the reference's state dictionaries.
"""

from __future__ import annotations

import ctypes as C
from typing import Any, Mapping

import numpy as np
import torch

from . import _lib
from .errors import MpasConfigError, MpasUnsupportedCapabilityError

# carried state keys (reference names) <-> field names
STATE_KEYS = ("u", "v", "ru", "ruAvg", "pv_edge", "w", "rw", "wwAvg", "theta_m", "rho_zz",
              "rho_p", "rtheta_p", "rtheta_base", "exner", "exner_base", "pressure_p",
              "pressure_base", "divergence", "ke", "rt_diabatic_tend", "uReconstructX",
              "uReconstructY", "uReconstructZ", "uReconstructZonal", "uReconstructMeridional",
              "vorticity", "scalars")
ALIASES = {"rho_edge": "h_edge", "h_edge": "h_edge", "ur_cell": "uReconstructZonal",
           "vr_cell": "uReconstructMeridional"}


def _np(x) -> np.ndarray:
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy()
    return np.asarray(x)


def _int(x) -> int:
    return int(_np(x).reshape(-1)[0]) if not isinstance(x, (int, np.integer)) else int(x)


def _conn0(a, n_target: int, rows: int) -> np.ndarray:
    """1-based padded connectivity -> 0-based active rows; sentinels -> padding row index."""
    a = _np(a).astype(np.int64)[:rows]
    return np.where((a >= 1) & (a <= n_target), a - 1, n_target).astype(np.int32)


class DeviceMesh:
    """Static mesh arrays on the device plus the ``mpasg_mesh`` struct that points at them."""

    def __init__(self, ref: Mapping[str, Any], device: torch.device | str = "cuda"):
        self.device = torch.device(device)
        nc, ne, nv = _int(ref["nCells"]), _int(ref["nEdges"]), _int(ref["nVertices"])
        nl = _int(ref["nVertLevels"])
        me = _int(ref["maxEdges"])
        me2 = _int(ref["maxEdges2"])
        vd = _int(ref["vertexDegree"])
        self.nCells, self.nEdges, self.nVertices, self.nVertLevels = nc, ne, nv, nl
        self.maxEdges, self.maxEdges2, self.vertexDegree = me, me2, vd
        adv = _np(ref["advCellsForEdge"])
        self.nAdvMax = int(adv.shape[1])
        self._keep: dict[str, torch.Tensor] = {}
        kite = _np(ref["kiteForCell"]).astype(np.int64)[:nc, :me]
        ints = {
            "nEdgesOnCell": _np(ref["nEdgesOnCell"]).astype(np.int32)[:nc],
            "edgesOnCell": _conn0(ref["edgesOnCell"], ne, nc)[:, :me],
            "cellsOnCell": _conn0(ref["cellsOnCell"], nc, nc)[:, :me],
            "verticesOnCell": _conn0(ref["verticesOnCell"], nv, nc)[:, :me],
            "kiteForCell": np.where((kite >= 1) & (kite <= vd), kite - 1, -1).astype(np.int32),
            "cellsOnEdge": _conn0(ref["cellsOnEdge"], nc, ne),
            "verticesOnEdge": _conn0(ref["verticesOnEdge"], nv, ne),
            "nEdgesOnEdge": _np(ref["nEdgesOnEdge"]).astype(np.int32)[:ne],
            "edgesOnEdge": _conn0(ref["edgesOnEdge"], ne, ne)[:, :me2],
            "nAdvCellsForEdge": _np(ref["nAdvCellsForEdge"]).astype(np.int32)[:ne],
            "advCellsForEdge": _conn0(ref["advCellsForEdge"], nc, ne),
            "edgesOnVertex": _conn0(ref["edgesOnVertex"], ne, nv)[:, :vd],
        }
        # slots beyond nEdgesOnCell / nEdgesOnEdge / nAdvCellsForEdge are never read
        dbls = {}
        a, a3 = _np(ref["adv_coefs"]).astype(np.float64), _np(ref["adv_coefs_3rd"]).astype(np.float64)
        derived = {"adv_coefs_p": a + a3, "adv_coefs_m": a - a3}
        derived.update(reference_theta_profile(_np(ref["theta_base"])[:nc, :nl].astype(np.float64),
                                               _np(ref["fzm"])[:nl].astype(np.float64),
                                               _np(ref["fzp"])[:nl].astype(np.float64)))
        for name in _lib.MESH_DBL_PTRS:
            if name in derived:
                dbls[name] = np.ascontiguousarray(derived[name])
                continue
            if name not in ref:
                raise MpasConfigError(f"mesh is missing {name}")
            dbls[name] = np.ascontiguousarray(_np(ref[name]), dtype=np.float64)
        if dbls["weightsOnEdge"].shape[1] > me2:
            dbls["weightsOnEdge"] = dbls["weightsOnEdge"][:, :me2]
        for key in ("edgesOnCell_sign", "defc_a", "defc_b"):
            dbls[key] = dbls[key][:, :me]
        dbls["coeffs_reconstruct"] = dbls["coeffs_reconstruct"][:, :me, :]
        dbls["zb_cell"] = dbls["zb_cell"][:, :me, :]
        dbls["zb3_cell"] = dbls["zb3_cell"][:, :me, :]
        for k in ("rdzw", "rdzu", "fzm", "fzp", "fnm", "fnp", "rdnw"):
            dbls[k] = dbls[k][:nl]
        st = _lib.MeshStruct()
        for n in ("nCells", "nEdges", "nVertices", "nVertLevels", "maxEdges", "maxEdges2",
                  "vertexDegree", "nAdvMax"):
            setattr(st, n, getattr(self, n))
        for n in _lib.MESH_F32_PTRS:  # float32 geometry of the mixed form
            t = torch.from_numpy(np.ascontiguousarray(dbls[n[:-4]], dtype=np.float32)).to(self.device)
            self._keep[n] = t
            setattr(st, n, t.data_ptr())
        st.flatTerrain = int(not np.any(dbls["zb_cell"]) and not np.any(dbls["zb3_cell"])
                             and not np.any(dbls["zxu"]))
        self.flat_terrain = bool(st.flatTerrain)
        for n in _lib.MESH_DOUBLES:
            setattr(st, n, float(_np(ref[n]).reshape(-1)[0]))
        for n, a in ints.items():
            t = torch.from_numpy(np.ascontiguousarray(a)).to(self.device)
            self._keep[n] = t
            setattr(st, n, t.data_ptr())
        # the acoustic flux sums' divergence weight, formed once: sign * dvEdge * invAreaCell
        eoc0 = ints["edgesOnCell"].astype(np.int64)
        geo = np.zeros((nc + 1, me))
        geo[:nc] = (dbls["edgesOnCell_sign"][:nc] * dbls["dvEdge"][np.minimum(eoc0, ne)]) * \
            dbls["invAreaCell"][:nc, None]
        dbls["cell_edge_geo"] = np.ascontiguousarray(geo)
        # per-slot products formed in the kernels' own association (bit-identical)
        ec = np.minimum(eoc0, ne)
        sg, dv, idc, ia = dbls["edgesOnCell_sign"][:nc], dbls["dvEdge"][ec], dbls["invDcEdge"][ec], \
            dbls["invAreaCell"][:nc, None]
        derived_slots = {"cell_edge_sdv": sg * dv, "cell_edge_es_w": (((0.5 * ia) * sg) * dv) * idc,
                         "cell_edge_es_t": ((ia * sg) * dv) * idc}
        for n, v in derived_slots.items():
            a = np.zeros((nc + 1, me))
            a[:nc] = v
            dbls[n] = a
        vd = self.vertexDegree
        eov0 = np.minimum(ints["edgesOnVertex"].astype(np.int64), ne)
        sdc = np.zeros((nv + 1, vd))
        sdc[:nv] = dbls["edgesOnVertex_sign"][:nv, :vd] * dbls["dcEdge"][eov0]
        derived_slots["vertex_edge_sdc"] = sdc
        dbls["vertex_edge_sdc"] = sdc
        dcdv = np.zeros(ne + 1)
        dcdv[:ne] = dbls["dcEdge"][:ne] * dbls["dvEdge"][:ne]
        derived_slots["edge_dcdv"] = dcdv
        dbls["edge_dcdv"] = dcdv
        lat, lon = _np(ref["latCell"]).astype(np.float64)[:nc], _np(ref["lonCell"]).astype(np.float64)[:nc]
        trig = np.zeros((nc + 1, 4))
        trig[:nc] = np.stack([np.cos(lat), np.sin(lat), np.cos(lon), np.sin(lon)], -1)
        derived_slots["cell_trig"] = trig
        dbls["cell_trig"] = trig
        for n in _lib.MESH_TAIL_PTRS:
            if n == "cell_edge_geo" or n in derived_slots:
                continue
            if n not in ref:
                raise MpasConfigError(f"mesh is missing {n}")
            a = _np(ref[n])
            a = a[:, :nl + 1] if n == "zgrid" else a[:nl] if a.ndim == 1 and n != "angleEdge" else a
            dbls[n] = np.ascontiguousarray(a, dtype=np.float64)
        for n, a in dbls.items():
            t = torch.from_numpy(np.ascontiguousarray(a)).to(self.device)
            self._keep[n] = t
            setattr(st, n, t.data_ptr())
        self.struct = st
        self.ints = ints


def reference_theta_profile(theta_base: np.ndarray, fzm: np.ndarray, fzp: np.ndarray) -> dict:
    """Per-level reference theta of the mixed form (the base-state theta of the first cell:
    any profile near theta works, and this one does not depend on how many cells follow,
    so an ensemble member gets the same profile alone and in a union) and its
    vertical-flux interface weights (the flux3 / second-order interpolations of
    kern_tend.cu applied to the profile)."""
    ref = theta_base[0].copy()
    nl = ref.shape[0]
    w4, w3, w2 = np.zeros(nl + 1), np.zeros(nl + 1), np.zeros(nl + 1)
    for k in range(1, nl):
        w2[k] = fzm[k] * ref[k] + fzp[k] * ref[k - 1]
    for k in range(2, nl - 1):
        w4[k] = (7.0 * (ref[k] + ref[k - 1]) - (ref[k + 1] + ref[k - 2])) / 12.0
        w3[k] = ((ref[k + 1] - ref[k - 2]) - 3.0 * (ref[k] - ref[k - 1])) / 12.0
    return {"ref_theta": ref, "ref_theta_w4": w4, "ref_theta_w3": w3, "ref_theta_w2": w2}


FIELD_KIND = dict(_lib.FIELDS)
ENTITY = {"e": "edge", "es": "edge", "c": "cell", "cw": "cell", "cs": "cell", "cws": "cell", "v": "vertex"}

ROWS = {"e": lambda m: (m.nEdges + 1, m.nVertLevels),
        "c": lambda m: (m.nCells + 1, m.nVertLevels),
        "cw": lambda m: (m.nCells + 1, m.nVertLevels + 1),
        "v": lambda m: (m.nVertices + 1, m.nVertLevels),
        "L": lambda m: (m.nVertLevels,)}


class DeviceState:
    """All device fields of one model instance (state, step work arrays and scratch)."""

    def __init__(self, mesh: DeviceMesh, num_scalars: int, only: frozenset | None = None):
        """``only``: allocate just these fields (a derivative state whose kernels touch no
        others; every other member of the C struct is a null pointer, and no float32
        copies are kept)."""
        self.mesh = mesh
        self.num_scalars = int(num_scalars)
        if not 0 <= self.num_scalars <= 8:
            raise MpasUnsupportedCapabilityError("0 to 8 scalars are supported")
        S = self.num_scalars
        shapes = dict((k, f(mesh)) for k, f in ROWS.items())
        shapes["cs"] = (mesh.nCells + 1, mesh.nVertLevels, S)
        shapes["es"] = (mesh.nEdges + 1, mesh.nVertLevels, S)
        shapes["cws"] = (mesh.nCells + 1, mesh.nVertLevels + 1, S)
        fields = [(n, k) for n, k in _lib.FIELDS if only is None or n in only]
        sizes = {name: int(np.prod(shapes[kind])) for name, kind in fields}
        total = sum(sizes.values())
        # one arena; each field is a contiguous view (256-byte aligned)
        align = 32
        offs = {}
        pos = 0
        for name, _ in fields:
            offs[name] = pos
            pos += (sizes[name] + align - 1) // align * align
        self.arena = torch.zeros(pos, dtype=torch.float64, device=mesh.device)
        self.f: dict[str, torch.Tensor] = {}
        st = _lib.FieldsStruct()
        for name, kind in fields:
            view = self.arena[offs[name]:offs[name] + sizes[name]].view(shapes[kind])
            self.f[name] = view
            setattr(st, name, view.data_ptr())
        # float32 members (mixed form), one float32 arena
        fields32 = _lib.FIELDS32 if only is None else []
        sizes32 = {name: int(np.prod(shapes[kind])) for name, kind in fields32}
        offs32, pos32 = {}, 0
        for name, _ in fields32:
            offs32[name] = pos32
            pos32 += (sizes32[name] + 63) // 64 * 64
        self.arena32 = torch.zeros(pos32, dtype=torch.float32, device=mesh.device)
        for name, kind in fields32:
            view = self.arena32[offs32[name]:offs32[name] + sizes32[name]].view(shapes[kind])
            self.f[name] = view
            setattr(st, name, view.data_ptr())
        self.status = torch.zeros(4, dtype=torch.int32, device=mesh.device)
        st.status = self.status.data_ptr()
        self.struct = st
        self.bytes = total * 8 + pos32 * 4
        # rho_zz padding row holds 1.0 (the reference's sentinel)
        if "rho_zz" in self.f:
            self.f["rho_zz"][mesh.nCells].fill_(1.0)
        # staging of loads that are gathered into the device order; reused field after
        # field (all on one stream), grown to the largest field
        self._stage = torch.empty(0, dtype=torch.float64, device=mesh.device)

    def field(self, name: str) -> torch.Tensor:
        return self.f[ALIASES.get(name, name)]

    def gather_rows(self, src: torch.Tensor, rows: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """out[i] = src[rows[i]] along the first dimension (``mpasg_permute_rows``)."""
        src = src.contiguous()
        out = torch.empty_like(src) if out is None else out
        lib = _lib.load()
        rc = lib.mpasg_permute_rows(C.c_void_p(src.data_ptr()), C.c_void_p(out.data_ptr()),
                                    C.c_void_p(rows.data_ptr()), int(src.shape[0]), int(src[0].numel()),
                                    C.c_void_p(torch.cuda.current_stream(src.device).cuda_stream))
        _lib.check(rc, "mpasg_permute_rows")
        return out

    def load(self, state: Mapping[str, Any], keys=None, rows: Mapping[str, torch.Tensor] | None = None,
             pending: dict | None = None) -> None:
        """Copy reference-layout arrays (numpy or torch) into the named fields; with
        ``rows`` (entity -> device row index, N+1 entries) the rows are gathered into the
        device order on the device, through one staging buffer kept across fields and
        calls.  ``pending`` maps a host tensor's address to the event of a device-to-host
        copy still writing it: the copy out of that tensor waits for that event only."""
        cur = torch.cuda.current_stream(self.mesh.device)
        for key in keys if keys is not None else state.keys():
            if key not in state:
                continue
            name = ALIASES.get(key, key)
            if name not in self.f:
                continue
            src = state[key]
            if not isinstance(src, (np.ndarray, torch.Tensor)):
                continue
            dst = self.f[name]
            if dst.numel() == 0:  # a model without scalars ignores the scalars it is given
                continue
            t = torch.as_tensor(src, dtype=torch.float64)
            if pending and isinstance(src, torch.Tensor):
                ev = pending.pop(src.data_ptr(), None)
                if ev is not None:
                    cur.wait_event(ev)
            ent = ENTITY.get(FIELD_KIND.get(name)) if rows is not None else None
            if ent is not None:
                if t.dim() != dst.dim() or tuple(t.shape[1:]) != tuple(dst.shape[1:]) or \
                        t.shape[0] not in (dst.shape[0], dst.shape[0] - 1):
                    raise MpasConfigError(f"{key}: shape {tuple(t.shape)} != {tuple(dst.shape)}")
                if self._stage.numel() < dst.numel():
                    self._stage = torch.empty(dst.numel(), dtype=torch.float64, device=dst.device)
                stage = self._stage[: dst.numel()].view(dst.shape)
                if t.shape[0] < stage.shape[0]:
                    stage[t.shape[0]:].zero_()
                stage[: t.shape[0]].copy_(t, non_blocking=True)
                self.gather_rows(stage, rows[ent], out=dst)
                continue
            if tuple(t.shape) != tuple(dst.shape):
                if t.dim() == dst.dim() and t.shape[0] == dst.shape[0] - 1:
                    dst[: t.shape[0]].copy_(t, non_blocking=True)
                    continue
                raise MpasConfigError(f"{key}: shape {tuple(t.shape)} != {tuple(dst.shape)}")
            dst.copy_(t, non_blocking=True)

    def export(self, keys=STATE_KEYS) -> dict[str, torch.Tensor]:
        out = {k: self.f[k] for k in keys}
        out["rho_edge"] = self.f["h_edge"]
        out["h_edge"] = self.f["h_edge"]
        out["ur_cell"] = self.f["uReconstructZonal"]
        out["vr_cell"] = self.f["uReconstructMeridional"]
        return out
