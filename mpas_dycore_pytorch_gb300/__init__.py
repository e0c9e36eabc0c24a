"""GB300 (sm_103a) implementation of MPAS-PyTorch's split-explicit dynamics timestep.

Drop-in for the reference's ``atm_srk3`` hot path (NOAA-EMC/mpas-dycore-pytorch,
``mpas_pytorch/dynamics/time_integration.py:4897``): the same padded state/mesh
dictionaries and key names, ``run_simulation`` / ``run_timestep`` / ``atm_srk3`` entry
points, computed by hand-written CUDA kernels in ``libmpasg.so`` (C ABI in
``include/mpasg.h``) on one GPU.  There is no CPU fallback.
"""

from .errors import (MpasConfigError, MpasDeviceError, MpasError, MpasExtensionMissingError,
                     MpasNumericalError, MpasUnsupportedCapabilityError)

__all__ = ["MpasConfigError", "MpasDeviceError", "MpasError", "MpasExtensionMissingError",
           "MpasNumericalError", "MpasUnsupportedCapabilityError", "run_simulation",
           "run_timestep", "atm_srk3", "Model"]


def __getattr__(name):
    if name in ("run_simulation", "run_timestep", "atm_srk3", "Model"):
        from . import api
        return getattr(api, name)
    raise AttributeError(name)
