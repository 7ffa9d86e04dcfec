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
    """pix2depth as a differentiable op of the vertex positions: apply(vtx2xyz,
    pix2tri, tri2vtx, transform_ndc2world) -> (img_h, img_w) depth.  The
    forward and the vertex gradient are the two kernels above; pix2tri, the
    triangles and the camera are constants of the op (no gradient)."""

    @staticmethod
    def forward(ctx, vtx2xyz, pix2tri, tri2vtx, transform_ndc2world):
        out = torch.zeros(tuple(pix2tri.shape), dtype=torch.float32, device=vtx2xyz.device)
        update(out, pix2tri, tri2vtx, vtx2xyz.detach(), transform_ndc2world)
        # the camera and the hit map are not differentiated, only replayed
        ctx.save_for_backward(vtx2xyz, pix2tri, tri2vtx, transform_ndc2world)
        return out

    @staticmethod
    def backward(ctx, grad_depth):
        vtx2xyz, pix2tri, tri2vtx, transform_ndc2world = ctx.saved_tensors
        if not ctx.needs_input_grad[0]:
            return None, None, None, None
        grad_vtx = vtx2xyz.new_zeros(vtx2xyz.shape)
        bwd_wrt_vtx2xyz(grad_vtx, pix2tri, tri2vtx, vtx2xyz.detach(), grad_depth.contiguous(), transform_ndc2world)
        return grad_vtx, None, None, None


def pix2depth_using_interpolation(vtx2xyz, pix2tri, tri2vtx, transform_ndc2world):
    """The depth of each pixel's hit point, differentiable in vtx2xyz: the
    function of the reference helper of this name, which interpolates the hit
    position from the vertex positions and projects it to ndc.  The hit point
    of a pixel's ray on its triangle is that interpolated position, so the
    fused depth kernel computes the same function and its gradient directly
    (one kernel each way, the world->ndc inverse on the device)."""
    return AutogradFunction.apply(vtx2xyz, pix2tri, tri2vtx, transform_ndc2world)
