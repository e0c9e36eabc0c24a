"""Reference runs at the benchmark's own sizes, stored as compact fixtures.

* ``full_c0``: the CPU-runnable case -- level-4 mesh (2562 cells x 26 levels), seed 0, 8 bumps, one
  cosine-bell tracer, non-monotone transport, dt 1800 s, 6 steps; the state after steps 2
  and 6;
* ``full_c1``: the headline case -- level-6 mesh (40962 cells x 55 levels, lowest layer 50 m), seed
  1, 32 bumps, 3 monotone tracers, dt 720 s; the state after 2 and 96 steps.

The arrays are too large to commit whole, so each field is stored as every ``stride``-th
row of the case (the last active row always included) at full precision, with its full active-row
sum of squares and a SHA-256 of its active rows (little-endian float64).  The loaded
connectivity's digests are stored too, and the SHA-256 of every raw array of the synthetic
case (``cases.make_case``, float arrays as little-endian float64), so that a run on another
machine can check it starts from the very inputs the reference started from.

Writes ``full_<case>.npz`` and ``full_<case>.json``.  Imports the reference as
``make_golden.py`` does (netCDF4 stub, ``MPAS_REFERENCE``).

Run:  MPAS_REFERENCE=<reference tree> python tests/golden/make_golden_full.py [case ...]
"""

from __future__ import annotations

import hashlib
import json
import os
import pathlib
import sys
import time

import numpy as np

os.environ["PYTHONDONTWRITEBYTECODE"] = "1"
os.environ.setdefault("ATEN_CPU_CAPABILITY", "default")

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent))

import make_golden  # noqa: E402

CASES = {
    "c0": dict(spec=dict(level=4, nlev=26, seed=0, n_bumps=8, n_tracers=1),
               config=dict(config_monotonic=False), dt=1800.0, steps=(2, 6), stride=37),
    "c1": dict(spec=dict(level=6, nlev=55, dz_bottom=50.0, seed=1, n_bumps=32, n_tracers=3),
               config=dict(config_monotonic=True), dt=720.0, steps=(2, 96), stride=211),
}
FIELDS = ("u", "w", "theta_m", "rho_zz", "scalars", "pressure_p", "exner", "rho_p", "rtheta_p", "ru", "rw", "v",
          "divergence", "vorticity", "ke", "pv_edge", "rho_edge")
CONNECTIVITY = ("cellsOnEdge", "edgesOnCell", "verticesOnEdge", "edgesOnVertex", "cellsOnCell", "edgesOnEdge",
                "nEdgesOnCell", "nEdgesOnEdge", "advCellsForEdge")


def active_rows(name, a, dims):
    n = {"u": "nEdges", "ru": "nEdges", "v": "nEdges", "pv_edge": "nEdges", "rho_edge": "nEdges",
         "vorticity": "nVertices"}.get(name, "nCells")
    return a[: dims[n]]


def sample_rows(n, stride):
    idx = np.arange(0, n, stride)
    if idx[-1] != n - 1:
        idx = np.append(idx, n - 1)
    return idx


def digest(a):
    a = np.ascontiguousarray(a, dtype="<f8")
    return hashlib.sha256(a.tobytes()).hexdigest()


def case_digests(init, grid):
    """SHA-256 of every array of the raw case (init/... and grid/...)."""
    out = {}
    for tag, d in (("init", init), ("grid", grid)):
        for k, v in sorted(d.items()):
            if isinstance(v, np.ndarray):
                a = np.ascontiguousarray(v, dtype="<f8" if v.dtype.kind == "f" else "<i8")
                out[f"{tag}/{k}"] = hashlib.sha256(a.tobytes()).hexdigest()
    return out


def record(out, meta, tag, state, dims, stride):
    for k in FIELDS:
        if k not in state:
            continue
        a = active_rows(k, state[k].detach().numpy(), dims)
        idx = sample_rows(a.shape[0], stride)
        out[f"{tag}/{k}/rows"] = idx
        out[f"{tag}/{k}/values"] = a[idx].copy()
        meta.setdefault(tag, {})[k] = {"sumsq": float(np.sum(a * a)), "sha256": digest(a), "shape": list(a.shape)}


def main() -> None:
    import torch
    mp = make_golden._import_reference()
    for name in sys.argv[1:] or list(CASES):
        case = CASES[name]
        state, mesh, cfg = make_golden.load_reference_case(mp, dict(case, nsteps=max(case["steps"])))
        dims = {k: int(mesh[k]) for k in ("nCells", "nEdges", "nVertices", "nVertLevels")}
        meta = {"case": name, "spec": case["spec"], "config": {k: v for k, v in cfg.items() if not k.startswith("_")},
                "dt": case["dt"], "steps": list(case["steps"]), "dims": dims, "stride": case["stride"],
                "torch": torch.__version__,
                "connectivity_sha256": {k: digest(np.asarray(mesh[k].numpy() if hasattr(mesh[k], "numpy") else mesh[k],
                                                              dtype=np.float64)) for k in CONNECTIVITY if k in mesh}}
        from mpas_dycore_pytorch_gb300.cases import CaseSpec, make_case
        meta["case_sha256"] = case_digests(*make_case(CaseSpec(**case["spec"])))
        out = {}
        want = set(case["steps"])
        t0 = time.time()

        def on_step(i, s):
            if i in want:
                record(out, meta, f"step{i}", s, dims, case["stride"])
                print(f"{name}: step {i} recorded at {time.time() - t0:.0f} s", flush=True)

        mp.run_simulation(state, mesh, config=cfg, dt=case["dt"], nsteps=max(case["steps"]), on_step=on_step)
        meta["seconds"] = time.time() - t0
        np.savez_compressed(HERE / f"full_{name}.npz", **out)
        (HERE / f"full_{name}.json").write_text(json.dumps(meta, indent=1, default=str))
        print(f"{name}: {meta['seconds']:.0f} s, {(HERE / f'full_{name}.npz').stat().st_size / 1e6:.1f} MB")


if __name__ == "__main__":
    main()
