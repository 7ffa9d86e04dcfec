"""Per-pixel closest-hit triangle by BVH ray casting on CUDA tensors.

Mirrors ``del_msh_dlpack/Pix2Tri/torch.py:8-61`` (by_raycasting).  Pixel
(iw, ih) casts the ray of ray_for_pixel.h through ``transform_ndc2world``
(row-major 4x4, transposed to column-major for the kernel as the reference
does); hits follow del-msh-cpu's search_bvh3::first_intersection_ray.
"""
from __future__ import annotations

from typing import Tuple

import torch

from .. import _native
from ..util_torch import assert_shape_dtype_device, ptr, require_cuda, scratch, stream_ptr


def by_raycasting(tri2vtx: torch.Tensor, vtx2xyz: torch.Tensor, bvhnodes: torch.Tensor, bvhnode2aabb: torch.Tensor,
                  transform_ndc2world: torch.Tensor, img_shape: Tuple[int, int], return_depth: bool = False):
    """Returns pix2tri (img_h, img_w) uint32 (u32::MAX where nothing is hit);
    with return_depth also pix2t (img_h, img_w) float32, the ray coefficient of
    the hit (+inf on a miss)."""
    vtx2xyz = vtx2xyz.detach()
    transform_ndc2world = transform_ndc2world.contiguous()
    num_tri, num_vtx, num_bvhnode = tri2vtx.shape[0], vtx2xyz.shape[0], bvhnodes.shape[0]
    device = tri2vtx.device
    assert num_bvhnode == num_tri * 2 - 1
    assert_shape_dtype_device(tri2vtx, (num_tri, 3), torch.uint32, device)
    assert_shape_dtype_device(vtx2xyz, (num_vtx, 3), torch.float32, device)
    assert_shape_dtype_device(bvhnodes, (num_bvhnode, 3), torch.uint32, device)
    assert_shape_dtype_device(bvhnode2aabb, (num_bvhnode, 6), torch.float32, device)
    assert_shape_dtype_device(transform_ndc2world, (4, 4), torch.float32, device)
    require_cuda(device)
    img_w, img_h = img_shape
    pix2tri = torch.empty((img_h, img_w), dtype=torch.uint32, device=device)
    pix2t = torch.empty((img_h, img_w), dtype=torch.float32, device=device) if return_depth else None
    colmajor = transform_ndc2world.T.contiguous()
    scr = scratch(device, _native.load().dm_cast_scratch_bytes(img_w * img_h, num_tri))
    _native.call("dm_pix2tri_by_raycast", stream_ptr(device), img_w, img_h, ptr(pix2tri), ptr(pix2t), num_tri,
                 ptr(tri2vtx.contiguous()), num_vtx, ptr(vtx2xyz.contiguous()), ptr(bvhnodes.contiguous()),
                 ptr(bvhnode2aabb.contiguous()), ptr(colmajor), ptr(scr), scr.numel())
    return (pix2tri, pix2t) if return_depth else pix2tri


def interpolate_fwd(pix2tri: torch.Tensor, tri2vtx: torch.Tensor, vtx2xyz: torch.Tensor, vtx2val: torch.Tensor,
                    transform_ndc2world: torch.Tensor):
    """pix2val (img_h, img_w, num_vdim): the vertex values interpolated with the
    barycentric coordinates of each pixel's ray on its triangle, 0 on the
    background (``del_msh_dlpack/Pix2Tri/torch.py`` interpolate_fwd)."""
    vtx2xyz, vtx2val = vtx2xyz.detach(), vtx2val.detach()
    num_tri, num_vtx, num_vdim = tri2vtx.shape[0], vtx2xyz.shape[0], vtx2val.shape[1]
    img_h, img_w = pix2tri.shape[0], pix2tri.shape[1]
    device = tri2vtx.device
    assert_shape_dtype_device(pix2tri, (img_h, img_w), torch.uint32, device)
    assert_shape_dtype_device(tri2vtx, (num_tri, 3), torch.uint32, device)
    assert_shape_dtype_device(vtx2xyz, (num_vtx, 3), torch.float32, device)
    assert_shape_dtype_device(vtx2val, (num_vtx, num_vdim), torch.float32, device)
    assert_shape_dtype_device(transform_ndc2world, (4, 4), torch.float32, device)
    require_cuda(device)
    pix2val = torch.zeros((img_h, img_w, num_vdim), dtype=torch.float32, device=device)
    _native.call("dm_pix2tri_interpolate", stream_ptr(device), img_w, img_h, ptr(pix2tri.contiguous()), num_tri,
                 ptr(tri2vtx.contiguous()), num_vtx, ptr(vtx2xyz.contiguous()), num_vdim, ptr(vtx2val.contiguous()),
                 ptr(transform_ndc2world.T.contiguous()), ptr(pix2val))
    return pix2val


def interpolate_bwd(pix2tri: torch.Tensor, tri2vtx: torch.Tensor, vtx2xyz: torch.Tensor, vtx2val: torch.Tensor,
                    transform_ndc2world: torch.Tensor, dldw_pix2val: torch.Tensor, dldw_vtx2xyz: torch.Tensor,
                    dldw_vtx2val: torch.Tensor):
    """Adds the backward of interpolate_fwd into dldw_vtx2xyz and dldw_vtx2val."""
    num_tri, num_vtx, num_vdim = tri2vtx.shape[0], vtx2xyz.shape[0], vtx2val.shape[1]
    img_h, img_w = pix2tri.shape[0], pix2tri.shape[1]
    device = tri2vtx.device
    assert_shape_dtype_device(pix2tri, (img_h, img_w), torch.uint32, device)
    assert_shape_dtype_device(tri2vtx, (num_tri, 3), torch.uint32, device)
    assert_shape_dtype_device(vtx2xyz, (num_vtx, 3), torch.float32, device)
    assert_shape_dtype_device(vtx2val, (num_vtx, num_vdim), torch.float32, device)
    assert_shape_dtype_device(transform_ndc2world, (4, 4), torch.float32, device)
    assert_shape_dtype_device(dldw_pix2val, (img_h, img_w, num_vdim), torch.float32, device)
    assert_shape_dtype_device(dldw_vtx2xyz, (num_vtx, 3), torch.float32, device)
    assert_shape_dtype_device(dldw_vtx2val, (num_vtx, num_vdim), torch.float32, device)
    require_cuda(device)
    _native.call("dm_pix2tri_interpolate_bwd", stream_ptr(device), img_w, img_h, ptr(pix2tri.contiguous()), num_tri,
                 ptr(tri2vtx.contiguous()), num_vtx, ptr(vtx2xyz.detach().contiguous()), num_vdim,
                 ptr(vtx2val.detach().contiguous()), ptr(transform_ndc2world.T.contiguous()),
                 ptr(dldw_pix2val.contiguous()), ptr(dldw_vtx2xyz), ptr(dldw_vtx2val))


class AutogradInterpolate(torch.autograd.Function):
    """Differentiable interpolation of vertex values as a torch.autograd.Function."""

    @staticmethod
    def forward(ctx, pix2tri, tri2vtx, vtx2xyz, vtx2val, transform_ndc2world):
        ctx.save_for_backward(pix2tri, tri2vtx, vtx2xyz, vtx2val, transform_ndc2world)
        return interpolate_fwd(pix2tri, tri2vtx, vtx2xyz, vtx2val, transform_ndc2world)

    @staticmethod
    def backward(ctx, dldw_pix2val):
        pix2tri, tri2vtx, vtx2xyz, vtx2val, transform_ndc2world = ctx.saved_tensors
        dldw_vtx2xyz = torch.zeros_like(vtx2xyz)
        dldw_vtx2val = torch.zeros_like(vtx2val)
        interpolate_bwd(pix2tri, tri2vtx, vtx2xyz.detach(), vtx2val.detach(), transform_ndc2world,
                        dldw_pix2val.contiguous(), dldw_vtx2xyz, dldw_vtx2val)
        return None, None, dldw_vtx2xyz, dldw_vtx2val, None


def interpolate(pix2tri, tri2vtx, vtx2xyz, vtx2val, transform_ndc2world):
    return AutogradInterpolate.apply(pix2tri, tri2vtx, vtx2xyz, vtx2val, transform_ndc2world)
