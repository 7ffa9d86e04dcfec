"""Closest hit of explicit rays on CUDA tensors: del-msh-cpu's
``search_bvh3::first_intersection_ray`` (search_bvh3.rs:103-221) applied to
every ray of an array."""
from __future__ import annotations

import torch

from .. import _native
from ..util_torch import assert_shape_dtype_device, ptr, require_cuda, scratch, stream_ptr


def first_intersection_ray(ray_org: torch.Tensor, ray_dir: torch.Tensor, tri2vtx: torch.Tensor,
                           vtx2xyz: torch.Tensor, bvhnodes: torch.Tensor, bvhnode2aabb: torch.Tensor,
                           return_bc: bool = False):
    """Returns (hit_tri (n,) uint32 [u32::MAX on a miss], hit_t (n,) float32
    [+inf on a miss]) and, with return_bc, barycentrics (n, 3) float32."""
    num_ray = ray_org.shape[0]
    num_tri, num_vtx, num_bvhnode = tri2vtx.shape[0], vtx2xyz.shape[0], bvhnodes.shape[0]
    device = tri2vtx.device
    assert num_bvhnode == num_tri * 2 - 1
    assert_shape_dtype_device(ray_org, (num_ray, 3), torch.float32, device)
    assert_shape_dtype_device(ray_dir, (num_ray, 3), torch.float32, device)
    assert_shape_dtype_device(tri2vtx, (num_tri, 3), torch.uint32, device)
    assert_shape_dtype_device(vtx2xyz, (num_vtx, 3), torch.float32, device)
    assert_shape_dtype_device(bvhnodes, (num_bvhnode, 3), torch.uint32, device)
    assert_shape_dtype_device(bvhnode2aabb, (num_bvhnode, 6), torch.float32, device)
    require_cuda(device)
    hit_tri = torch.empty((num_ray,), dtype=torch.uint32, device=device)
    hit_t = torch.empty((num_ray,), dtype=torch.float32, device=device)
    hit_bc = torch.empty((num_ray, 3), dtype=torch.float32, device=device) if return_bc else None
    scr = scratch(device, _native.load().dm_cast_scratch_bytes(num_ray, num_tri))
    _native.call("dm_search_bvh3_first_intersection_ray", stream_ptr(device), num_ray,
                 ptr(ray_org.detach().contiguous()), ptr(ray_dir.detach().contiguous()), ptr(hit_tri), ptr(hit_t),
                 ptr(hit_bc), num_tri, ptr(tri2vtx.contiguous()), num_vtx, ptr(vtx2xyz.detach().contiguous()),
                 ptr(bvhnodes.contiguous()), ptr(bvhnode2aabb.contiguous()), ptr(scr), scr.numel())
    return (hit_tri, hit_t, hit_bc) if return_bc else (hit_tri, hit_t)
