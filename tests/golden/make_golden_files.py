"""The reference's own load_initial_state on the MPAS grid / initial-condition files this
package writes (cases.write_case_files, NetCDF-3 with the MPAS schema).

For the level-2 case of g2_explicit and the level-4 CPU-runnable case: write the two files,
load them with the reference's unmodified ``load_initial_state(init_path, grid_path)``
(its CheckpointReader over make_golden's read-only netCDF4 stand-in, the netCDF4 package
being absent here), and record the SHA-256 of both files and of every array the reference
returns (state and mesh), with its shape and, for float arrays, its sum of squares.

Writes ``files_<case>.json``.  Imports the reference as ``make_golden.py`` does
(``MPAS_REFERENCE``).

Run:  MPAS_REFERENCE=<reference tree> python tests/golden/make_golden_files.py
"""

from __future__ import annotations

import hashlib
import json
import os
import pathlib
import sys
import tempfile

import numpy as np

os.environ["PYTHONDONTWRITEBYTECODE"] = "1"
os.environ.setdefault("ATEN_CPU_CAPABILITY", "default")

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent))

import make_golden  # noqa: E402

CASES = {
    "g2": dict(spec=make_golden.CASES["g2_explicit"]["spec"], config=make_golden.CASES["g2_explicit"]["config"],
               dt=make_golden.CASES["g2_explicit"]["dt"]),
    "c0": dict(spec=dict(level=4, nlev=26, seed=0, n_bumps=8, n_tracers=1), config=dict(config_monotonic=False),
               dt=1800.0),
}


def digest(a: np.ndarray) -> str:
    a = np.ascontiguousarray(a, dtype="<f8" if a.dtype.kind == "f" else "<i8")
    return hashlib.sha256(a.tobytes()).hexdigest()


def record(d) -> dict:
    out = {}
    for k, v in sorted(d.items()):
        if hasattr(v, "detach"):
            a = v.detach().cpu().numpy()
            out[k] = {"sha256": digest(a), "shape": list(a.shape), "kind": a.dtype.kind}
            if a.dtype.kind == "f":
                out[k]["sumsq"] = float(np.sum(a.astype(np.float64) ** 2))
    return out


def main() -> None:
    import torch
    mp = make_golden._import_reference(make_golden._READER_STUB)
    from mpas_dycore_pytorch_gb300.cases import CaseSpec, write_case_files
    for name, case in CASES.items():
        cfg = dict(make_golden.BASE_CONFIG)
        cfg.update(case["config"])
        cfg["config_dt"] = case["dt"]
        tmp = pathlib.Path(tempfile.mkdtemp(prefix=f"case_{name}_"))
        init_path, grid_path = write_case_files(CaseSpec(**case["spec"]), tmp)
        state, mesh = mp.load_initial_state(init_path, grid_path, config=cfg)
        meta = {"case": name, "spec": case["spec"], "config": cfg, "torch": torch.__version__,
                "files_sha256": {p.name: hashlib.sha256(p.read_bytes()).hexdigest() for p in (init_path, grid_path)},
                "state": record(state), "mesh": record(mesh)}
        (HERE / f"files_{name}.json").write_text(json.dumps(meta, indent=1))
        print(f"{name}: {len(meta['state'])} state and {len(meta['mesh'])} mesh arrays from "
              f"{', '.join(meta['files_sha256'])}")


if __name__ == "__main__":
    main()
