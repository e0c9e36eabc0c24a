"""Typed errors with the reference's ``MpasError`` hierarchy (mpas_pytorch/exceptions.py:30-154).

As in the reference, every configuration-side error is an ``MpasConfigError`` (a
``ValueError``): unsupported capabilities, unavailable devices, missing fields, mesh
mismatches, strict-mode rejections.  C-ABI status codes map onto these types in
``_lib.check``.
"""

from __future__ import annotations

from typing import Iterable


class MpasError(Exception):
    """Base class of every error this package raises."""


class MpasConfigError(MpasError, ValueError):
    """Invalid configuration, shapes or inputs (reference: exceptions.MpasConfigError)."""


class MpasProvenanceError(MpasConfigError):
    """A derived field was supplied from outside where it must be computed."""


class MpasMissingFieldError(MpasConfigError):
    """Required initial-condition or mesh fields are absent."""

    def __init__(self, message: str | None = None, *, fields: Iterable[str] | None = None,
                 source: str = "unknown") -> None:
        self.fields = tuple(fields or ())
        self.source = str(source)
        if message is None and self.fields:
            message = f"Missing required fields from {self.source}: {self.fields}"
        super().__init__(message if message is not None else "")


class MpasMeshMismatchError(MpasConfigError):
    """Initial-condition and mesh dimensions disagree."""

    def __init__(self, message: str | None = None, *, dim_name: str | None = None,
                 init_value: int | None = None, grid_value: int | None = None) -> None:
        self.dim_name, self.init_value, self.grid_value = dim_name, init_value, grid_value
        if message is None and dim_name is not None:
            message = f"Mesh dimension mismatch for {dim_name}: init={init_value}, grid={grid_value}"
        super().__init__(message if message is not None else "")


class MpasStrictModeError(MpasConfigError):
    """Strict validation rejected an unknown or unwired setting."""


class MpasUnsupportedCapabilityError(MpasConfigError, NotImplementedError):
    """A requested option is outside the supported path (reference: same name)."""


class MpasDeviceError(MpasConfigError, RuntimeError):
    """The device is unavailable, or a CUDA runtime / launch failure."""

    def __init__(self, message: str | None = None, *, requested: str | None = None) -> None:
        self.requested = "" if requested is None else str(requested)
        if message is None and self.requested:
            message = f"{self.requested!r} requested but no CUDA device is visible; the GB300 path runs on CUDA only"
        super().__init__(message if message is not None else "")


class MpasNumericalError(MpasConfigError):
    """Non-finite model fields (the reference raises MpasConfigError for these)."""


class MpasNumericalAgreementError(MpasError):
    """A numerical-agreement contract failed (reference: same name)."""


class MpasExtensionMissingError(MpasDeviceError, ImportError):
    """``libmpasg.so`` is not built; the device path has no CPU fallback."""
