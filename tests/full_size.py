"""Helpers for the benchmark-size fixtures made by tests/golden/make_golden_full.py."""

from __future__ import annotations

import functools
import hashlib
import json
import pathlib

import numpy as np

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
BASE_CONFIG = {"config_time_integration_order": 3, "config_len_disp": 120000.0,
               "config_number_of_sub_steps": 2, "config_dynamics_split_steps": 3}
EDGE_FIELDS = ("u", "ru", "v", "pv_edge", "rho_edge")


@functools.lru_cache(maxsize=None)
def fixture(case: str):
    meta = json.loads((GOLDEN / f"full_{case}.json").read_text())
    arrays = dict(np.load(GOLDEN / f"full_{case}.npz"))
    return meta, arrays


def config(meta) -> dict:
    cfg = dict(BASE_CONFIG)
    cfg.update({k: v for k, v in meta["config"].items() if k in ("config_monotonic",)})
    cfg["config_dt"] = float(meta["dt"])
    return cfg


def sha256_f64(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(np.asarray(a, dtype=np.float64), dtype="<f8").tobytes()).hexdigest()


def active(name: str, a: np.ndarray, dims) -> np.ndarray:
    n = dims["nEdges"] if name in EDGE_FIELDS else dims["nVertices"] if name == "vorticity" else dims["nCells"]
    return a[:n]


def case_digest_mismatches(meta) -> list[str]:
    """Raw case arrays (cases.make_case on this machine) whose SHA-256 differs from the one
    recorded beside the reference run: the run would not start from the reference's inputs."""
    from mpas_dycore_pytorch_gb300.cases import CaseSpec, make_case
    init, grid = make_case(CaseSpec(**meta["spec"]))
    got = {}
    for tag, d in (("init", init), ("grid", grid)):
        for k, v in d.items():
            if isinstance(v, np.ndarray):
                a = np.ascontiguousarray(v, dtype="<f8" if v.dtype.kind == "f" else "<i8")
                got[f"{tag}/{k}"] = hashlib.sha256(a.tobytes()).hexdigest()
    want = meta["case_sha256"]
    return sorted(k for k in set(want) | set(got) if want.get(k) != got.get(k))

