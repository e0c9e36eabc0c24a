"""Every CUDA stage entry point against the reference's own stage calls (golden taps)."""

import numpy as np
import pytest

from fixtures import CASES, rel_l2, tap_calls
from gpu_helpers import model_for_case, need_gpu, to_np
from oracle.step import stage_names

pytestmark = pytest.mark.gpu

KEYS = ("moist", "vimp", "dyn_tend", "smlstep", "acoustic", "divdamp", "recover", "diag",
        "scalars", "scalars_mono", "reconstruct")
# float64 with fused multiply-add on the GPU vs the reference's unfused CPU arithmetic
TOL = 1e-12
# rthdynten is a diagnostic output (physics coupling) formed as a difference of nearly
# equal tendencies; its relative error is that cancellation times the roundoff above
TOL_BY_NAME = {"rthdynten": 1e-10}
# In the moist case's second and third RK stages the horizontal theta flux divergence nearly
# cancels: one-ulp noise on the stage inputs moves tend_theta by 1.7e-12 in the oracle itself
TOL_BY_CASE_NAME = {("g2_moist", "tend_theta"): 5e-12}


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("key", KEYS)
def test_cuda_stage_matches_reference(case, key):
    need_gpu()
    from mpas_dycore_pytorch_gb300.stages import STAGES, run_stage
    calls = [call for name in stage_names(key) for call in tap_calls(case, name)]
    if not calls:
        pytest.skip("stage not called in this case")
    model, meta, st, mesh = model_for_case(case)
    outputs = STAGES[key][3]
    for inp, ref_out, entry in calls:
        got = run_stage(model, key, inp)
        for name in outputs:
            if name not in ref_out:
                continue
            r = np.asarray(ref_out[name])
            g = to_np(got[name])
            if g.shape != r.shape:
                assert g.shape[0] == r.shape[0] + 1, (name, g.shape, r.shape)
                g = g[:-1]
            n = {inp.get("nCells"), inp.get("nEdges"), inp.get("nVertices")}
            rows = r.shape[0] - 1 if (r.shape[0] - 1) in n else r.shape[0]
            err = rel_l2(g[:rows], r[:rows])
            tol = TOL_BY_CASE_NAME.get((case, name), TOL_BY_NAME.get(name, TOL))
            assert err <= tol, (key, entry["index"], name, err)
