"""Typed errors, mirroring the reference's ``MpasError`` hierarchy (mpas_pytorch/exceptions.py:30-154).

``MpasConfigError`` subclasses ``ValueError`` as in the reference; C-ABI status codes map
onto these types in ``_lib.check``.
"""


class MpasError(Exception):
    """Base class of every error this package raises."""


class MpasConfigError(MpasError, ValueError):
    """Invalid configuration, shapes or inputs (reference: exceptions.MpasConfigError)."""


class MpasUnsupportedCapabilityError(MpasError, NotImplementedError):
    """A requested option is outside the supported path (reference: same name)."""


class MpasDeviceError(MpasError, RuntimeError):
    """CUDA runtime or launch failure (reference: exceptions.MpasDeviceError)."""


class MpasNumericalError(MpasConfigError):
    """Non-finite model fields (the reference raises MpasConfigError for these)."""


class MpasExtensionMissingError(MpasDeviceError, ImportError):
    """``libmpasg.so`` is not built; the device path has no CPU fallback."""
