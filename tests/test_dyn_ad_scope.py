"""Host-side checks of the dynamics derivatives' device state: the cotangent state allocates
only COTANGENT_FIELDS, so that list must hold every field the reverse-mode kernels name."""

import pathlib
import re

from mpas_dycore_pytorch_gb300 import _lib
from mpas_dycore_pytorch_gb300.dyn_adjoint import CARRIED, COTANGENT_FIELDS

CSRC = pathlib.Path(__file__).resolve().parent.parent / "mpas_dycore_pytorch_gb300" / "csrc"
REVERSE_SOURCES = ("kern_adj_column.cu", "kern_adj_tend.cu", "kern_adj_diag.cu", "driver_adj.cu")


def test_cotangent_fields_cover_every_field_the_reverse_kernels_name():
    fields = {n for n, _ in _lib.FIELDS} | {n for n, _ in _lib.FIELDS32}
    named = set()
    for name in REVERSE_SOURCES:
        text = (CSRC / name).read_text()
        named |= {m for m in re.findall(r"\bg(?:\.|->)(\w+)", text) if m in fields}
    missing = named - COTANGENT_FIELDS
    assert not missing, sorted(missing)
    assert set(CARRIED) <= COTANGENT_FIELDS
    assert COTANGENT_FIELDS <= {n for n, _ in _lib.FIELDS}
