"""Shared helpers for the GPU parity tests (CUDA path vs golden fixtures and the oracle)."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from fixtures import group, load_case


def need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")


def model_for_case(case: str, num_scalars=None, precision=None):
    from mpas_dycore_pytorch_gb300.api import Model
    meta, st, _ = load_case(case)
    loaded = group(st, "loaded")
    mesh = dict(loaded)
    mesh.update(meta["loaded_scalars"])
    ns = num_scalars or int(loaded["scalars"].shape[-1])
    return Model(mesh, meta["config"], meta["dt"], num_scalars=ns, precision=precision), meta, st, mesh


def to_np(x):
    return x.detach().cpu().numpy() if isinstance(x, torch.Tensor) else np.asarray(x)
