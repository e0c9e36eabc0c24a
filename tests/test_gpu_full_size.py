"""The float64 GPU path against the reference itself at the benchmark's own sizes
(tests/golden/make_golden_full.py): the CPU-runnable case (level-4 mesh, 2562 cells x 26
levels, 6 steps) and the headline case (level-6 mesh, 40962 cells x 55 levels, 3 monotone
tracers, 96 steps).  The run starts from the reference run's very inputs (the generated
case's digests are checked first).  Each recorded field is compared on the fixture's
sampled rows (relative L2) and by its full-field norm, against the stated 1e-12 for every
field, after 2 steps and at the end of the run alike.  Measured on GB300: level 4 <= 1.1e-13
after 2 steps and <= 1.3e-13 after 6; level 6 <= 1.3e-13 after 2 steps and <= 1.8e-13 after
96 (w and rw the largest)."""

import numpy as np
import pytest
import torch

from fixtures import STEP_TOL
from full_size import GOLDEN, active, case_digest_mismatches, config, fixture
from gpu_helpers import need_gpu

pytestmark = pytest.mark.gpu



@pytest.mark.parametrize("case", ("c0", "c1"))
def test_state_matches_reference_at_benchmark_size(case):
    need_gpu()
    if not (GOLDEN / f"full_{case}.json").exists():
        pytest.skip("fixture not generated")
    from mpas_dycore_pytorch_gb300.api import run_simulation
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.loader import load_case
    meta, arr = fixture(case)
    bad = case_digest_mismatches(meta)
    assert not bad, f"the generated case differs from the reference run's input: {bad[:5]}"
    cfg = config(meta)
    st, _ = load_case(CaseSpec(**meta["spec"]), cfg, as_torch=True)
    dims = meta["dims"]
    steps = set(meta["steps"])
    got = {}

    def on_step(i, s):
        if i not in steps:
            return
        for k in meta[f"step{i}"]:
            a = active(k, s[k], dims)
            rows = torch.as_tensor(arr[f"step{i}/{k}/rows"], device=a.device)
            got[(i, k)] = (a.index_select(0, rows).cpu().numpy(), float((a.double() ** 2).sum()))

    run_simulation(st, st, cfg, float(meta["dt"]), nsteps=max(steps), on_step=on_step)
    worst = {}
    for (i, k), (vals, sumsq) in sorted(got.items()):
        ref = arr[f"step{i}/{k}/values"]
        den = np.linalg.norm(ref)
        err = np.linalg.norm(vals - ref) / (den if den > 0 else 1.0)
        ref_norm = np.sqrt(meta[f"step{i}"][k]["sumsq"])
        nerr = abs(np.sqrt(sumsq) - ref_norm) / (ref_norm if ref_norm > 0 else 1.0)
        print(f"{case} step {i} {k}: sampled rel L2 {err:.2e}, norm rel {nerr:.2e}")
        worst[(i, k)] = max(err, nerr)
    assert len(got) == sum(len(meta[f"step{i}"]) for i in steps)
    fails = [(i, k, e) for (i, k), e in worst.items() if e > STEP_TOL]
    assert not fails, fails
