"""Depth image from a pix2tri map, forward and backward, on CUDA tensors.

Mirrors ``del_msh_dlpack/Pix2Depth/torch.py`` (update, bwd_wrt_vtx2xyz,
AutogradFunction, pix2depth_using_interpolation): depth = (ndc z + 1) / 2 of
the hit point of each pixel's ray on its triangle, 0 on the background
(CPU ``pix2depth.rs:107-146``, GPU ``pix2depth.cu``).  The world->ndc
inverse is computed on the device, with no host round trip.
"""
from __future__ import annotations

import torch

from .. import _native
from ..util_torch import assert_shape_dtype_device, ptr, require_cuda, stream_ptr


def _scratch(device) -> torch.Tensor:
    """Room for the device-side world->ndc matrix, from torch's caching
    allocator (256-byte aligned)."""
    return torch.empty((_native.load().dm_render_scratch_bytes(),), dtype=torch.uint8, device=device)


def update(pix2depth: torch.Tensor, pix2tri: torch.Tensor, tri2vtx: torch.Tensor, vtx2xyz: torch.Tensor,
           transform_ndc2world: torch.Tensor):
    """Writes the depth of every pixel into pix2depth (img_h, img_w) float32."""
    num_tri, num_vtx = tri2vtx.shape[0], vtx2xyz.shape[0]
    img_h, img_w = pix2depth.shape[0], pix2depth.shape[1]
    device = pix2depth.device
    assert_shape_dtype_device(pix2depth, (img_h, img_w), torch.float32, device)
    assert_shape_dtype_device(pix2tri, (img_h, img_w), torch.uint32, device)
    assert_shape_dtype_device(tri2vtx, (num_tri, 3), torch.uint32, device)
    assert_shape_dtype_device(vtx2xyz, (num_vtx, 3), torch.float32, device)
    assert_shape_dtype_device(transform_ndc2world, (4, 4), torch.float32, device)
    require_cuda(device)
    colmajor = transform_ndc2world.T.contiguous()
    scratch = _scratch(device)
    _native.call("dm_pix2depth_update", stream_ptr(device), img_w, img_h, ptr(pix2depth), ptr(pix2tri.contiguous()),
                 num_tri, ptr(tri2vtx.contiguous()), num_vtx, ptr(vtx2xyz.detach().contiguous()), ptr(colmajor),
                 ptr(scratch), scratch.numel())


def bwd_wrt_vtx2xyz(dldw_vtx2xyz: torch.Tensor, pix2tri: torch.Tensor, tri2vtx: torch.Tensor, vtx2xyz: torch.Tensor,
                    dldw_pix2depth: torch.Tensor, transform_ndc2world: torch.Tensor):
    """Adds d(depth)/d(vtx2xyz)^T dldw_pix2depth into dldw_vtx2xyz (num_vtx, 3)."""
    num_tri, num_vtx = tri2vtx.shape[0], vtx2xyz.shape[0]
    img_h, img_w = pix2tri.shape[0], pix2tri.shape[1]
    device = dldw_vtx2xyz.device
    assert_shape_dtype_device(dldw_vtx2xyz, (num_vtx, 3), torch.float32, device)
    assert_shape_dtype_device(pix2tri, (img_h, img_w), torch.uint32, device)
    assert_shape_dtype_device(tri2vtx, (num_tri, 3), torch.uint32, device)
    assert_shape_dtype_device(vtx2xyz, (num_vtx, 3), torch.float32, device)
    assert_shape_dtype_device(dldw_pix2depth, (img_h, img_w), torch.float32, device)
    assert_shape_dtype_device(transform_ndc2world, (4, 4), torch.float32, device)
    require_cuda(device)
    colmajor = transform_ndc2world.T.contiguous()
    scratch = _scratch(device)
    _native.call("dm_pix2depth_bwd_wrt_vtx2xyz", stream_ptr(device), img_w, img_h, ptr(dldw_vtx2xyz),
                 ptr(pix2tri.contiguous()), num_tri, ptr(tri2vtx.contiguous()), num_vtx,
                 ptr(vtx2xyz.detach().contiguous()), ptr(dldw_pix2depth.contiguous()), ptr(colmajor), ptr(scratch),
                 scratch.numel())


class AutogradFunction(torch.autograd.Function):
    """Differentiable depth rendering as a torch.autograd.Function."""

    @staticmethod
    def forward(ctx, vtx2xyz, pix2tri, tri2vtx, transform_ndc2world):
        ctx.save_for_backward(pix2tri, tri2vtx, vtx2xyz, transform_ndc2world)
        pix2depth = torch.zeros(pix2tri.shape, dtype=torch.float32, device=vtx2xyz.device)
        update(pix2depth, pix2tri, tri2vtx, vtx2xyz.detach(), transform_ndc2world)
        return pix2depth

    @staticmethod
    def backward(ctx, dldw_pix2depth):
        pix2tri, tri2vtx, vtx2xyz, transform_ndc2world = ctx.saved_tensors
        dldw_vtx2xyz = torch.zeros_like(vtx2xyz)
        bwd_wrt_vtx2xyz(dldw_vtx2xyz, pix2tri, tri2vtx, vtx2xyz.detach(), dldw_pix2depth.contiguous(),
                        transform_ndc2world)
        return dldw_vtx2xyz, None, None, None


def pix2depth_using_interpolation(vtx2xyz, pix2tri, tri2vtx, transform_ndc2world):
    """Depth through the interpolated hit position (differentiable through
    Pix2Tri.AutogradInterpolate)."""
    from ..Pix2Tri.torch import AutogradInterpolate
    pix2xyz = AutogradInterpolate.apply(pix2tri, tri2vtx, vtx2xyz, vtx2xyz, transform_ndc2world)
    transform_world2ndc = transform_ndc2world.inverse()
    pix2xyzw = torch.cat([pix2xyz, torch.ones_like(pix2xyz[:, :, :1])], dim=-1)
    background = pix2tri == torch.iinfo(torch.uint32).max
    pix2ndcw = pix2xyzw @ transform_world2ndc.T
    pix2depth = (pix2ndcw[:, :, 2] / pix2ndcw[:, :, 3] + 1.0) * 0.5
    pix2depth[background] = 0.0
    return pix2depth
