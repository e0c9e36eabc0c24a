"""Loader for the golden fixtures made by ``tests/golden/make_golden.py``."""

from __future__ import annotations

import functools
import json
import pathlib

import numpy as np

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
CASES = ("g2_explicit", "g2_mono", "g2_moist", "g2_rk2", "g2_fixed", "g2_cam", "g2_split2", "g2_coupled",
         "g2_rayleigh", "g2_posdef", "g2_noadv")

# Bound on the relative L2 difference of a field after whole large steps.  w and rw come
# out of the vertically implicit acoustic solve, whose right-hand side is the small
# difference of the vertical pressure gradient and buoyancy; pow() (the Exner function)
# rounds its last bit differently in different math libraries, and cancellation amplifies
# that.  One-ulp noise injected into the oracle's exner moves w / rw after one step by
# 1.5e-12 / 1.7e-12 (g2_explicit), 4.4e-12 / 7.1e-12 (g2_rk2), 4.0e-12 / 4.9e-12 (g2_cam),
# 3.6e-12 / 5.0e-12 (g2_posdef), 3.1e-12 / 3.8e-12 (g2_noadv), 2.1e-12 / 2.2e-12 (g2_split2),
# while every stage taken alone is bit-identical to the reference apart from pow().  So w
# and rw are bound at 1e-11 and every other field at 1e-12.
STEP_TOL = 1e-12
STEP_TOL_VERTICAL = 1e-11


def step_tol(case: str, field: str) -> float:
    if field in ("w", "rw"):
        return STEP_TOL_VERTICAL
    return STEP_TOL


@functools.lru_cache(maxsize=None)
def load_case(name: str):
    meta = json.loads((GOLDEN / f"{name}.json").read_text())
    state = dict(np.load(GOLDEN / f"{name}_state.npz"))
    taps = dict(np.load(GOLDEN / f"{name}_taps.npz"))
    return meta, state, taps


def group(state: dict, prefix: str) -> dict:
    p = prefix + "/"
    return {k[len(p):]: v for k, v in state.items() if k.startswith(p)}


def tap_calls(name: str, stage: str):
    """Yield ``(inputs, outputs, entry)`` for every recorded call of ``stage``."""
    meta, state, taps = load_case(name)
    loaded = group(state, "loaded")
    for entry in meta["taps"]:
        if entry["stage"] != stage:
            continue
        pre = f"{stage}/{entry['index']}"
        inp = {k: loaded[k] for k in entry["static_in"]}
        for k in entry["arrays_in"]:
            inp[k] = taps[f"{pre}/in/{k}"]
        for k, v in entry["scalars"].items():
            if not k.startswith("out:"):
                inp[k] = v
        out = {k: taps[f"{pre}/out/{k}"] for k in entry["arrays_out"]}
        yield inp, out, entry


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b.ravel())
    num = np.linalg.norm((a - b).ravel())
    if den == 0.0:
        return float(num)
    return float(num / den)
