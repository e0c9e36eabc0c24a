"""mpasg_advance_scalars_static: transport with the library's own fixed edge scratch.

It must give exactly what mpasg_advance_scalars gives (same kernels, other scratch), leave
the caller's hflux alone (it may be null), and refuse problems larger than the scratch
before touching the device.  The file name sorts last so the GPU test also runs after
every other test in one session.
"""

import ctypes as C

import numpy as np
import pytest
import torch

from fixtures import CASES, tap_calls
from gpu_helpers import model_for_case, need_gpu
from oracle.step import stage_names


def test_oversize_problem_is_refused_before_any_device_work():
    from mpas_dycore_pytorch_gb300 import _lib
    from mpas_dycore_pytorch_gb300.build import build
    from mpas_dycore_pytorch_gb300.errors import MpasConfigError
    try:
        build()
    except RuntimeError as exc:  # no nvcc on this machine
        pytest.skip(str(exc))
    lib = _lib.load()
    m, c, f = _lib.MeshStruct(), _lib.ConfigStruct(), _lib.FieldsStruct()
    m.nCells, m.nEdges, m.nVertLevels = 40962, 122880, 55  # 120 km mesh, 55 levels
    c.num_scalars = 3
    assert m.nEdges * m.nVertLevels * c.num_scalars > _lib.STATIC_SCRATCH_DOUBLES
    rc = lib.mpasg_advance_scalars_static(C.byref(m), C.byref(c), C.byref(f), 1, 1.0, None)
    assert rc == -5
    with pytest.raises(MpasConfigError, match="static scratch"):
        _lib.check(rc, "mpasg_advance_scalars_static")


def _two_stage_calls(model, entry, inp, fields):
    """Two calls in a row from the tapped inputs: the second continues from the first."""
    from mpas_dycore_pytorch_gb300.stages import STAGES
    st = model.state
    for ref_name, field in STAGES["scalars"][2].items():
        if hasattr(inp.get(ref_name), "shape"):
            st.load({field: inp[ref_name]}, keys=(field,))
    fn = getattr(model.lib, entry)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    outs = []
    for rk in (int(inp["rk_step"]), int(inp["rk_step"]) + 1):
        rc = fn(C.byref(model.dmesh.struct), C.byref(model.cstruct), C.byref(fields),
                C.c_int(min(rk, 3)), C.c_double(float(inp["dt"])), stream)
        assert rc == 0, (entry, rc)
        outs.append(st.f["scalars_b"].clone())
        st.f["scalars_a"].copy_(st.f["scalars_b"])
    torch.cuda.current_stream().synchronize()
    return outs


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["float64", "mixed"])
@pytest.mark.parametrize("case", CASES)
def test_static_scratch_matches_caller_scratch_entry(case, precision):
    """Both instantiations of the transport kernels (float64 and the mixed form's float32
    stencils) write the library's scratch exactly as they write the caller's."""
    need_gpu()
    from mpas_dycore_pytorch_gb300 import _lib
    calls = [call for name in stage_names("scalars") for call in tap_calls(case, name)]
    if not calls:
        pytest.skip("no explicit transport stage in this case")
    inp = calls[0][0]
    model, _, _, _ = model_for_case(case, precision=precision)
    st = model.state
    want = _two_stage_calls(model, "mpasg_advance_scalars", inp, st.struct)
    # the static entry point gets no hflux at all; the caller's hflux must stay untouched
    st.f["hflux"].fill_(float("nan"))
    fields = _lib.FieldsStruct.from_buffer_copy(st.struct)
    fields.hflux = None
    got = _two_stage_calls(model, "mpasg_advance_scalars_static", inp, fields)
    for w, g in zip(want, got):
        assert torch.isfinite(g).all()
        assert torch.equal(w, g)
    assert torch.isnan(st.f["hflux"]).all()
    # second use on the same device (scratch address cached) gives the same again
    again = _two_stage_calls(model, "mpasg_advance_scalars_static", inp, fields)
    for w, g in zip(want, again):
        assert torch.equal(w, g)
    assert np.isfinite(want[1].cpu().numpy()).all()
