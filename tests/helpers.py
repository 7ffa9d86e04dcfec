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
    return np.ascontiguousarray(a).view(np.uint32)
