"""Algorithmic HBM byte model of one large step (v1).

Convention: each stage call compulsorily reads each distinct input field and writes each
output field once.  A field is counted in units of one (C x L) array: a cell or W-level
field is 1 unit, an edge field E/C ~ 3, a vertex field V/C ~ 2 and a per-slot cell metric
(C x maxEdges x (L+1)) 6.  Bookkeeping copies, zero fills and alias refreshes are excluded.

Per call (calls per large step with split = 3, RK3, ns = 2):
  moist 5+S [1]; vert_imp_coefs 16 [6]; dyn_tend 59 [9]; smlstep_pert 18 [9];
  acoustic + divergence damping 48 [12]; recover 51 [9]; solve_diagnostics 17 [9];
  explicit transport 6+3S [2, or 3 without the limiter]; monotone transport 6+13S [0 or 1];
  reconstruct 10 [1].
Total units U = 2010 + 10 S (non-monotone) or 2010 + 20 S (monotone); bytes per
cell-level-step = 8 U in float64.
"""

from __future__ import annotations

UNITS_PER_CALL = {
    "moist": lambda S: 5 + S,
    "vert_imp_coefs": lambda S: 16,
    "dyn_tend": lambda S: 59,
    "smlstep_pert": lambda S: 18,
    "acoustic_divdamp": lambda S: 48,
    "recover": lambda S: 51,
    "diagnostics": lambda S: 17,
    "scalars": lambda S: 6 + 3 * S,
    "scalars_mono": lambda S: 6 + 13 * S,
    "reconstruct": lambda S: 10,
}


def calls_per_step(split: int = 3, ns: int = 2, order: int = 3, monotonic: bool = True) -> dict:
    nsub = [1, max(ns // 2, 1), ns] if order == 3 else [max(ns // 2, 1), max(ns // 2, 1), ns]
    vimp = 2 if order == 3 else 1
    return {
        "moist": 1, "vert_imp_coefs": vimp * split, "dyn_tend": 3 * split,
        "smlstep_pert": 3 * split, "acoustic_divdamp": sum(nsub) * split,
        "recover": 3 * split, "diagnostics": 3 * split,
        "scalars": 2 if monotonic else 3, "scalars_mono": 1 if monotonic else 0,
        "reconstruct": 1,
    }


def units_per_step(S: int, monotonic: bool = True, **kw) -> int:
    calls = calls_per_step(monotonic=monotonic, **kw)
    return sum(UNITS_PER_CALL[k](S) * n for k, n in calls.items())


def bytes_per_cell_level_step(S: int, monotonic: bool = True, width: int = 8, **kw) -> int:
    return width * units_per_step(S, monotonic, **kw)


# Mixed form: units of each stage that its kernels read as float32 copies (4 B) instead of
# the float64 state (8 B).  dyn_tend reads u and pv_edge (edge fields, 3 units each), w and
# rw (W-level fields, 1 unit each) as float32; every other field, and every output, stays
# float64.  Stages not listed are counted in float64 (an upper bound).
MIXED_F32_UNITS = {"dyn_tend": 8}


def stage_bytes_per_call(stage: str, S: int, n_cells: int, n_levels: int, width: int = 8,
                         precision: str = "float64") -> int:
    units = UNITS_PER_CALL[stage](S)
    f32 = MIXED_F32_UNITS.get(stage, 0) if precision == "mixed" else 0
    return (width * (units - f32) + 4 * f32) * n_cells * n_levels
