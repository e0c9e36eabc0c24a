"""The benchmark-size cases (configs[0]: level-4 2562 x 26; configs[1]: level-6 40962 x 55)
as this package's loader builds them have the reference loader's connectivity bit for bit
(SHA-256 digests recorded by tests/golden/make_golden_full.py from the reference's own
load_initial_state)."""

import numpy as np
import pytest

from full_size import GOLDEN, config, fixture, sha256_f64


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
