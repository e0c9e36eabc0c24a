"""GB300 (sm_103a) implementation of MPAS-PyTorch's split-explicit dynamics timestep.

Drop-in for the reference's ``atm_srk3`` hot path (NOAA-EMC/mpas-dycore-pytorch,
``mpas_pytorch/dynamics/time_integration.py:4897``): the same padded state/mesh
dictionaries and key names, the reference's public names (``run_simulation`` with its
``.jvp`` / ``.vjp``, ``run_timestep``, the loaders and the error types), computed by
hand-written CUDA kernels in ``libmpasg.so`` (C ABI in ``include/mpasg.h``) on one GPU.
There is no CPU fallback.
"""

from .errors import (MpasConfigError, MpasDeviceError, MpasError, MpasExtensionMissingError,
                     MpasMeshMismatchError, MpasMissingFieldError, MpasNumericalAgreementError,
                     MpasNumericalError, MpasProvenanceError, MpasStrictModeError,
                     MpasUnsupportedCapabilityError)
from .loading import (load_config_from_namelist, load_initial_state, read_history, read_restart,
                      write_history, write_restart)

# the reference's public surface (mpas_pytorch.__all__), then this package's additions
REFERENCE_SURFACE = ("MpasConfigError", "MpasDeviceError", "MpasError", "MpasMeshMismatchError",
                     "MpasMissingFieldError", "MpasNumericalAgreementError", "MpasProvenanceError",
                     "MpasStrictModeError", "MpasUnsupportedCapabilityError", "load_config_from_namelist",
                     "load_initial_state", "read_history", "read_restart", "run_simulation", "run_timestep",
                     "write_history", "write_restart")
__all__ = list(REFERENCE_SURFACE) + ["MpasExtensionMissingError", "MpasNumericalError", "atm_srk3", "Model"]


def __getattr__(name):
    if name in ("run_simulation", "run_timestep", "atm_srk3", "Model"):
        from . import api
        return getattr(api, name)
    raise AttributeError(name)
