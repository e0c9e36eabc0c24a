"""The reference-named keyword operators (``work.py``) against the reference's own stage
calls (golden taps of g2_explicit and g2_mono): the reference's keyword arguments in, its
outputs with its names and shapes out, within the stage-parity bounds of
``test_gpu_stages.py``."""

import numpy as np
import pytest

from fixtures import group, load_case, rel_l2, tap_calls
from gpu_helpers import need_gpu, to_np
from oracle.step import stage_names

pytestmark = pytest.mark.gpu

TOL = 1e-12
TOL_BY_NAME = {"rthdynten": 1e-10}


@pytest.mark.parametrize("case", ("g2_explicit", "g2_mono"))
def test_keyword_operators_match_the_reference(case):
    need_gpu()
    from mpas_dycore_pytorch_gb300 import work
    meta, st, _ = load_case(case)
    mesh = dict(group(st, "loaded"))
    mesh.update(meta["loaded_scalars"])
    work.use_mesh(mesh, meta["config"], meta["dt"])
    checked = 0
    for routine, (key, _) in work.ROUTINES.items():
        for name in stage_names(key):
            for inp, ref_out, entry in list(tap_calls(case, name))[:2]:
                got = getattr(work, routine)(**inp)
                for out_name, r in ref_out.items():
                    if out_name not in got:
                        continue
                    r = np.asarray(r)
                    g = to_np(got[out_name])
                    assert g.shape == r.shape, (routine, out_name, g.shape, r.shape)
                    n = {inp.get("nCells"), inp.get("nEdges"), inp.get("nVertices")}
                    rows = r.shape[0] - 1 if (r.shape[0] - 1) in n else r.shape[0]
                    err = rel_l2(g[:rows], r[:rows])
                    assert err <= TOL_BY_NAME.get(out_name, TOL), (routine, entry["index"], out_name, err)
                    checked += 1
    assert checked > 50
