"""The reference's own gradient and tangent on the differentiation workload at its stated
size, stored compactly.

Workload: level-5 mesh (10242 cells x 41 levels), seed 2, 8 bumps, one passive tracer,
0.1 m/s sinusoidal w, wind rounded to 16 significant bits, RK3 with 3 dynamics substeps x 2
acoustic substeps, non-monotone transport, dt 900 s, 24 steps; functional J = sum_c
areaCell_c (sp_c(T) - sp_ref_c)^2 of the hydrostatic surface pressure (as in
make_golden_dyn_ad.py).  Recorded: ``run_simulation.vjp`` of J with respect to the
initial u and theta, ``run_simulation.jvp`` along a seeded direction (Box-Muller draws
from PCG64, cases._normal: the same on every machine; padding rows zero) for the final
rho_zz, pressure_p, u, theta_m and w, J and the reference surface pressure.  Each array is stored as every ``STRIDE``-th
active row plus the last, with its full sum of squares and SHA-256; the SHA-256 of every
generated input array is stored too.

Writes ``dyn_ad_c2.npz`` and ``dyn_ad_c2.json``.

Run:  MPAS_REFERENCE=<reference tree> python tests/golden/make_golden_dyn_ad_full.py
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
import make_golden_dyn_ad  # noqa: E402
import make_golden_full  # noqa: E402

CASE = dict(spec=dict(level=5, nlev=41, seed=2, n_bumps=8, n_tracers=1, w_sine=0.1, round_wind_bits=16),
            config=dict(config_monotonic=False), dt=900.0, nsteps=24)
STRIDE = 53
DIRECTION_SEED = 20261204
TRACK = make_golden_dyn_ad.TRACK
JVP_KEYS = make_golden_dyn_ad.JVP_KEYS


def direction(shapes: dict) -> dict:
    """The seeded perturbation of u (scale 1) and theta (scale 0.1), padding rows zero."""
    from mpas_dycore_pytorch_gb300.cases import _normal
    rng = np.random.default_rng(DIRECTION_SEED)
    out = {}
    for k in TRACK:
        d = _normal(rng, shapes[k]) * (1.0 if k == "u" else 0.1)
        d[-1] = 0.0
        out[k] = d
    return out


def compact(out, meta, tag, a):
    a = np.asarray(a, dtype=np.float64)
    n = a.shape[0] - 1  # active rows
    rows = make_golden_full.sample_rows(n, STRIDE)
    out[f"{tag}/rows"] = rows
    out[f"{tag}/values"] = a[rows].copy()
    meta[tag] = {"sumsq": float(np.sum(a[:n] ** 2)), "sha256": make_golden_full.digest(a[:n]),
                 "shape": list(a.shape)}


def main() -> None:
    import torch
    mp = make_golden._import_reference()
    from mpas_dycore_pytorch_gb300.cases import CaseSpec, make_case
    state, meshd, cfg = make_golden.load_reference_case(mp, CASE)
    dt, nsteps = CASE["dt"], CASE["nsteps"]

    def fresh():
        return make_golden.load_reference_case(mp, CASE)[:2]

    prepared = {}
    st_, me_ = fresh()
    mp.run_simulation(st_, me_, config=cfg, dt=dt, nsteps=1,
                      on_initial=lambda s: prepared.update({k: v.detach().clone() for k, v in s.items()
                                                           if isinstance(v, torch.Tensor)}))
    sp_fn, _ = make_golden_dyn_ad.objective_factory(mp, meshd, None)
    nc = int(meshd["nCells"])
    sp_ref = sp_fn(dict(prepared))[:nc].detach().clone()
    meta = {"spec": CASE["spec"], "config": cfg, "dt": dt, "nsteps": nsteps, "stride": STRIDE,
            "direction_seed": DIRECTION_SEED, "torch": torch.__version__,
            "case_sha256": make_golden_full.case_digests(*make_case(CaseSpec(**CASE["spec"])))}
    out: dict[str, np.ndarray] = {"sp_ref": sp_ref.numpy()}
    st_, me_ = fresh()
    _, objective = make_golden_dyn_ad.objective_factory(mp, me_, sp_ref)
    t0 = time.time()
    grads = mp.run_simulation.vjp(st_, me_, objective, track_keys=TRACK, config=cfg, dt=dt, nsteps=nsteps)
    meta["vjp_seconds"] = time.time() - t0
    print(f"vjp {meta['vjp_seconds']:.0f} s", flush=True)
    for k in TRACK:
        compact(out, meta, f"grad_{k}", grads[k].detach().numpy())
    st_, me_ = fresh()
    final = mp.run_simulation(st_, me_, config=cfg, dt=dt, nsteps=nsteps)
    _, objective = make_golden_dyn_ad.objective_factory(mp, me_, sp_ref)
    meta["J"] = float(objective(final))
    dirs = direction({k: tuple(state[k].shape) for k in TRACK})
    meta["direction_sha256"] = {k: make_golden_full.digest(v) for k, v in dirs.items()}
    st_, me_ = fresh()
    t0 = time.time()
    tang = mp.run_simulation.jvp(st_, me_, {k: torch.from_numpy(v) for k, v in dirs.items()},
                                 config=cfg, dt=dt, nsteps=nsteps)
    meta["jvp_seconds"] = time.time() - t0
    for k in JVP_KEYS:
        compact(out, meta, f"jvp_{k}", tang[k].detach().numpy())
    np.savez_compressed(HERE / "dyn_ad_c2.npz", **out)
    (HERE / "dyn_ad_c2.json").write_text(json.dumps(meta, indent=1, default=str))
    print(f"J = {meta['J']:.6e}, vjp {meta['vjp_seconds']:.0f} s, jvp {meta['jvp_seconds']:.0f} s, "
          f"{(HERE / 'dyn_ad_c2.npz').stat().st_size / 1e6:.1f} MB")


if __name__ == "__main__":
    main()
