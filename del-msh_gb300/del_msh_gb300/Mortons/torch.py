"""Morton codes and radix-tree topology on CUDA tensors.

Mirrors ``del_msh_dlpack/Mortons/torch.py`` (make_vtx2morton_from_vtx2co at
:5-46, make_bvhnodes_from_sorted_mortons at :49-82): same names, argument
meaning, output shapes and dtypes.
"""
from __future__ import annotations

import torch

from .. import _native
from ..util_torch import assert_shape_dtype_device, ptr, require_cuda, stream_ptr


def make_vtx2morton_from_vtx2co(vtx2co: torch.Tensor, transform_co2unit: torch.Tensor) -> torch.Tensor:
    """Morton code of each point after ``transform_co2unit`` (a row-major
    (d+1)x(d+1) matrix) maps it into the unit cube; coordinates outside
    [0,1] are clamped as del-msh-cpu does.

    Args:
        vtx2co: (num_vtx, 2 or 3) float32
        transform_co2unit: (3x3 or 4x4) float32
    Returns:
        vtx2morton: (num_vtx,) uint32
    """
    vtx2co = vtx2co.detach().contiguous()
    num_vtx, num_dim = vtx2co.shape
    device = vtx2co.device
    assert num_dim == 2 or num_dim == 3
    assert_shape_dtype_device(vtx2co, (num_vtx, num_dim), torch.float32, device)
    assert_shape_dtype_device(transform_co2unit, (num_dim + 1, num_dim + 1), torch.float32, device)
    require_cuda(device)
    vtx2morton = torch.empty((num_vtx,), device=device, dtype=torch.uint32)
    colmajor = transform_co2unit.detach().T.contiguous()
    _native.call("dm_mortons_vtx2morton_from_vtx2co", stream_ptr(device), num_vtx, num_dim, ptr(vtx2co),
                 ptr(colmajor), ptr(vtx2morton))
    return vtx2morton


def make_bvhnodes_from_sorted_mortons(idx2obj: torch.Tensor, idx2morton: torch.Tensor) -> torch.Tensor:
    """Binary radix tree over sorted Morton codes.

    Args:
        idx2obj: (n,) uint32 - object index of each sorted code
        idx2morton: (n,) uint32 - sorted Morton codes
    Returns:
        bvhnodes: (2n-1, 3) uint32 - [parent, left, right] per node
    """
    n = idx2obj.shape[0]
    device = idx2obj.device
    assert idx2obj.dtype == torch.uint32 and idx2obj.dim() == 1
    assert idx2morton.dtype == torch.uint32 and idx2morton.dim() == 1
    assert idx2obj.shape == idx2morton.shape
    require_cuda(device)
    bvhnodes = torch.empty((n * 2 - 1, 3), device=device, dtype=torch.uint32)
    _native.call("dm_mortons_make_bvhnodes_from_sorted_mortons", stream_ptr(device), n,
                 ptr(idx2obj.contiguous()), ptr(idx2morton.contiguous()), ptr(bvhnodes))
    return bvhnodes
