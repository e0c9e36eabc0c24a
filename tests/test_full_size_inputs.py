"""The benchmark-size cases (level-4 2562 x 26, the CPU-runnable case; level-6 40962 x 55,
the headline case): the synthetic case generator reproduces, bit for bit, the raw arrays the
reference run started from, and this package's loader builds the reference loader's
connectivity from them (SHA-256 digests recorded by tests/golden/make_golden_full.py)."""

import numpy as np
import pytest

from full_size import GOLDEN, case_digest_mismatches, config, fixture, sha256_f64


@pytest.mark.parametrize("case", ("c0", "c1"))
def test_connectivity_matches_the_reference_loader(case):
    if not (GOLDEN / f"full_{case}.json").exists():
        pytest.skip("fixture not generated")
    from mpas_dycore_pytorch_gb300.cases import CaseSpec
    from mpas_dycore_pytorch_gb300.loader import load_case
    meta, _ = fixture(case)
    st, _ = load_case(CaseSpec(**meta["spec"]), config(meta), as_torch=False)
    for k, d in meta["connectivity_sha256"].items():
        assert sha256_f64(st[k]) == d, k
    for k, n in meta["dims"].items():
        assert int(np.asarray(st[k])) == n, k


@pytest.mark.parametrize("case", ("c0", "c1"))
def test_generated_case_is_the_reference_runs_input(case):
    if not (GOLDEN / f"full_{case}.json").exists():
        pytest.skip("fixture not generated")
    meta, _ = fixture(case)
    assert not case_digest_mismatches(meta)

