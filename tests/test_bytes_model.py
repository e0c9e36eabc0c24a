"""The v1 algorithmic byte model (bytes_model.py): per-call units and the totals per
cell-level-step of the headline and CPU-runnable cases."""

from mpas_dycore_pytorch_gb300.bytes_model import (UNITS_PER_CALL, bytes_per_cell_level_step,
                                                   stage_bytes_per_call, units_per_step)


def test_units_per_step():
    # U = 2010 + 10 S (non-monotone) or 2010 + 20 S (monotone)
    for S in (0, 1, 3):
        assert units_per_step(S, monotonic=False) == 2010 + 10 * S
        assert units_per_step(S, monotonic=True) == 2010 + 20 * S
    assert bytes_per_cell_level_step(1, monotonic=False) == 16160
    assert bytes_per_cell_level_step(3, monotonic=True) == 16560


def test_stage_bytes_float64_and_mixed():
    C, L = 40962, 55
    assert stage_bytes_per_call("dyn_tend", 3, C, L) == 8 * UNITS_PER_CALL["dyn_tend"](3) * C * L
    # mixed: u, pv_edge (3 units each), w, rw (1 each) read as float32
    assert stage_bytes_per_call("dyn_tend", 3, C, L, precision="mixed") == (8 * 51 + 4 * 8) * C * L
    assert stage_bytes_per_call("recover", 3, C, L, precision="mixed") == stage_bytes_per_call("recover", 3, C, L)
