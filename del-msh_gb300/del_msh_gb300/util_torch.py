"""Helpers shared by the torch front-ends (the checks of
del_msh_dlpack/util_torch.py: shape, dtype and device assertions)."""
from __future__ import annotations

import torch


def assert_shape_dtype_device(t: torch.Tensor, shape, dtype, device):
    assert t.shape == tuple(shape), f"shape {tuple(t.shape)} != {tuple(shape)}"
    assert t.dtype == dtype, f"dtype {t.dtype} != {dtype}"
    assert t.device == device, f"device {t.device} != {device}"


def require_cuda(device: torch.device):
    if device.type != "cuda":
        raise NotImplementedError("del_msh_gb300 runs on CUDA devices only (no CPU path)")


def stream_ptr(device: torch.device) -> int:
    torch.cuda.set_device(device)
    return torch.cuda.current_stream(device).cuda_stream


def ptr(t):
    """Device address of a contiguous tensor (None -> NULL)."""
    if t is None:
        return None
    assert t.is_contiguous(), "tensor must be contiguous"
    return t.data_ptr()


def scratch(device: torch.device, nbytes: int) -> torch.Tensor:
    """Working memory for one C-ABI call, from torch's caching allocator (so
    repeated calls reuse it instead of allocating on the device each time);
    its blocks are 512-byte aligned, as the C ABI requires 256."""
    return torch.empty((max(int(nbytes), 1),), dtype=torch.uint8, device=device)
