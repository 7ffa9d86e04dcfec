"""numpy <-> torch helpers for the tests (uint32 goes through an int32 view)."""
import numpy as np


def to_dev(a, torch, device="cuda:0"):
    a = np.ascontiguousarray(a)
    if a.dtype == np.uint32:
        return torch.from_numpy(a.view(np.int32)).to(device).view(torch.uint32)
    return torch.from_numpy(a).to(device)


def to_np(t, torch):
    if t.dtype == torch.uint32:
        return t.view(torch.int32).cpu().numpy().view(np.uint32)
    return t.cpu().numpy()


def bits(a):
    """Raw bits for exact comparison; every NaN is mapped to one pattern (NaN
    payloads differ between x86, Arm and CUDA and carry no information here)."""
    a = np.array(a, copy=True)
    if a.dtype == np.float32:
        a[np.isnan(a)] = np.float32("nan")
    return np.ascontiguousarray(a).view(np.uint32)
