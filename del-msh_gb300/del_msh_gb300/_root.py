"""Shared plumbing of the package-root entry points (the DLPack-level
functions of del_msh_dlpack's sub-packages): tensors from DLPack objects and
scratch that is safe on the caller's stream."""
from __future__ import annotations

import torch


def as_tensor(x) -> torch.Tensor:
    """A torch tensor viewing x (a tensor, or anything torch.from_dlpack takes)."""
    t = x if isinstance(x, torch.Tensor) else torch.from_dlpack(x)
    if t.device.type != "cuda":
        raise NotImplementedError("del_msh_gb300 runs on CUDA devices only (no CPU path)")
    if not t.is_contiguous():
        raise ValueError("arrays must be contiguous")
    return t


def call_on_stream(stream_ptr: int, device: torch.device, scratch_bytes: int, fn):
    """Runs fn(scratch) for a launch on the raw CUDA stream stream_ptr.  The
    scratch comes from torch's caching allocator and is marked as used by that
    stream, so torch does not hand it out again before the launch is done."""
    with torch.cuda.device(device):
        scr = torch.empty((max(int(scratch_bytes), 1),), dtype=torch.uint8, device=device)
        fn(scr)
        cur = torch.cuda.current_stream(device)
        if int(stream_ptr) != cur.cuda_stream:
            scr.record_stream(torch.cuda.ExternalStream(int(stream_ptr), device=device) if stream_ptr
                              else torch.cuda.default_stream(device))
