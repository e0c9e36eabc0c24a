"""CPU oracle for the MPAS split-explicit dynamics step (numpy restatement).

TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` may import this package, and only as the
checker or the timed CPU baseline.  The product path (``mpas_dycore_pytorch_gb300``)
never imports it and fails loudly when its CUDA extension is missing.

The oracle restates the reference's float64 algorithm for the ``atm_srk3`` hot
path (NOAA-EMC/mpas-dycore-pytorch v0.1.7, ``mpas_pytorch/dynamics/*.py``) in
vectorised numpy, one function per reference stage, each citing the reference
function it follows.  It is pinned against golden fixtures produced by running
the reference itself (``tests/golden/make_golden.py``): per-stage inputs/outputs
of every stage call in one large step, and the full boundary after 1 and 2 steps.
"""

from .stages import *  # noqa: F401,F403
from .step import *  # noqa: F401,F403
