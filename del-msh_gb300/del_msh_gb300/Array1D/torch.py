"""Stable argsort of u32 arrays on CUDA tensors.

Mirrors ``del_msh_dlpack/Array1D/torch.py:41-70`` (argsort).
"""
from __future__ import annotations

import torch

from .. import _native
from ..util_torch import ptr, require_cuda, scratch, stream_ptr


def argsort(idx2val: torch.Tensor):
    """Sorted order of a 1D uint32 array; equal values keep ascending index.

    Args:
        idx2val: (n,) uint32
    Returns:
        jdx2idx: (n,) uint32 - original index of each sorted element
        jdx2val: (n,) uint32 - sorted values
    """
    n = idx2val.shape[0]
    device = idx2val.device
    assert idx2val.shape == (n,)
    assert idx2val.dtype == torch.uint32
    require_cuda(device)
    jdx2idx = torch.empty(size=(n,), device=device, dtype=torch.uint32)
    jdx2val = idx2val.clone()
    scr = scratch(device, _native.load().dm_array1d_argsort_scratch_bytes(n))
    _native.call("dm_array1d_argsort", stream_ptr(device), n, ptr(jdx2val), ptr(jdx2idx), ptr(scr), scr.numel())
    return jdx2idx, jdx2val
