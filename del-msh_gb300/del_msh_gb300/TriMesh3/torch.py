"""LBVH build and refit of triangle meshes on CUDA tensors.

Mirrors ``del_msh_dlpack/TriMesh3/torch.py:233-285``
(make_bvhnodes_bvhnode2aabb) and ``TriMesh3/__init__.py:39-46``
(make_bvhnode2aabb_from_bvhnodes -> bvhnode2aabb_update_aabb).  The results
are those of del-msh-cpu (bvhnodes_morton::from_triangle_mesh and
bvhnode2aabb3::from_uniform_mesh_with_bvh): centroids are (p0+p1+p2)*(1/3) in
f32 and the sort keeps equal codes in triangle order.
"""
from __future__ import annotations

import torch

from .. import _native
from ..util_torch import assert_shape_dtype_device, ptr, require_cuda, scratch, stream_ptr


def make_bvhnodes_bvhnode2aabb(tri2vtx: torch.Tensor, vtx2xyz: torch.Tensor):
    """LBVH of a triangle mesh.

    Args:
        tri2vtx: (num_tri, 3) uint32
        vtx2xyz: (num_vtx, 3) float32
    Returns:
        bvhnodes: (2*num_tri-1, 3) uint32 - [parent, left, right] per node
        bvhnode2aabb: (2*num_tri-1, 6) float32 - [min xyz, max xyz] per node
    """
    vtx2xyz = vtx2xyz.detach()
    num_vtx = vtx2xyz.shape[0]
    num_tri = tri2vtx.shape[0]
    device = tri2vtx.device
    assert_shape_dtype_device(tri2vtx, (num_tri, 3), torch.uint32, device)
    assert_shape_dtype_device(vtx2xyz, (num_vtx, 3), torch.float32, device)
    require_cuda(device)
    bvhnodes = torch.empty((2 * num_tri - 1, 3), dtype=torch.uint32, device=device)
    bvhnode2aabb = torch.empty((2 * num_tri - 1, 6), dtype=torch.float32, device=device)
    scr = scratch(device, _native.load().dm_trimesh3_build_scratch_bytes(num_tri))
    _native.call("dm_trimesh3_make_bvhnodes_bvhnode2aabb", stream_ptr(device), num_tri, ptr(tri2vtx.contiguous()),
                 num_vtx, ptr(vtx2xyz.contiguous()), ptr(bvhnodes), ptr(bvhnode2aabb), ptr(scr), scr.numel())
    return bvhnodes, bvhnode2aabb


def make_bvhnodes_bvhnode2aabb_ex(tri2vtx: torch.Tensor, vtx2xyz: torch.Tensor, want_height: bool = True):
    """The same build, also returning its intermediate values: a dict with
    bvhnodes, bvhnode2aabb, transform (4x4 row-major float32), tri2morton,
    idx2tri, idx2morton (uint32) and height (int, or None without
    want_height).  Asking for the height makes the refit climb the tree in
    tree order instead of answering range queries; the boxes are the same."""
    vtx2xyz = vtx2xyz.detach().contiguous()
    num_vtx, num_tri = vtx2xyz.shape[0], tri2vtx.shape[0]
    device = tri2vtx.device
    assert_shape_dtype_device(tri2vtx, (num_tri, 3), torch.uint32, device)
    assert_shape_dtype_device(vtx2xyz, (num_vtx, 3), torch.float32, device)
    require_cuda(device)
    out = dict(bvhnodes=torch.empty((2 * num_tri - 1, 3), dtype=torch.uint32, device=device),
               bvhnode2aabb=torch.empty((2 * num_tri - 1, 6), dtype=torch.float32, device=device),
               transform=torch.empty((16,), dtype=torch.float32, device=device),
               tri2morton=torch.empty((num_tri,), dtype=torch.uint32, device=device),
               idx2tri=torch.empty((num_tri,), dtype=torch.uint32, device=device),
               idx2morton=torch.empty((num_tri,), dtype=torch.uint32, device=device),
               height=torch.zeros((1,), dtype=torch.int32, device=device) if want_height else None)
    scr = scratch(device, _native.load().dm_trimesh3_build_scratch_bytes(num_tri))
    _native.call("dm_trimesh3_build_ex", stream_ptr(device), num_tri, ptr(tri2vtx.contiguous()), num_vtx,
                 ptr(vtx2xyz), ptr(out["bvhnodes"]), ptr(out["bvhnode2aabb"]), ptr(out["transform"]),
                 ptr(out["tri2morton"]), ptr(out["idx2tri"]), ptr(out["idx2morton"]),
                 ptr(out["height"]) if want_height else None, ptr(scr), scr.numel())
    out["transform"] = out["transform"].view(4, 4).T.contiguous()
    out["height"] = int(out["height"].item()) if want_height else None
    return out


def update_bvhnode2aabb(tri2vtx: torch.Tensor, vtx2xyz0: torch.Tensor, bvhnodes: torch.Tensor,
                        bvhnode2aabb: torch.Tensor, vtx2xyz1: torch.Tensor | None = None,
                        flags: torch.Tensor | None = None) -> torch.Tensor:
    """Refit: recompute every node AABB of an existing tree for (possibly
    deformed) vertices, in place.  With vtx2xyz1 the boxes enclose both
    positions (continuous collision detection).  ``flags`` is an optional
    persistent (num_tri-1,) uint32 zero buffer reused across calls."""
    num_tri = tri2vtx.shape[0]
    num_vtx = vtx2xyz0.shape[0]
    num_bvhnode = bvhnodes.shape[0]
    device = tri2vtx.device
    assert_shape_dtype_device(tri2vtx, (num_tri, 3), torch.uint32, device)
    assert_shape_dtype_device(vtx2xyz0, (num_vtx, 3), torch.float32, device)
    assert_shape_dtype_device(bvhnodes, (num_bvhnode, 3), torch.uint32, device)
    assert_shape_dtype_device(bvhnode2aabb, (num_bvhnode, 6), torch.float32, device)
    if vtx2xyz1 is not None and vtx2xyz1.shape[0] != num_vtx:
        vtx2xyz1 = None  # the binding ignores a second position array of another size
    if vtx2xyz1 is not None:
        assert_shape_dtype_device(vtx2xyz1, (num_vtx, 3), torch.float32, device)
    if flags is not None:
        assert flags.dtype == torch.uint32 and flags.numel() >= num_tri - 1
    require_cuda(device)
    _native.call("dm_bvhnode2aabb_update_aabb", stream_ptr(device), num_bvhnode, ptr(bvhnode2aabb), 0, ptr(bvhnodes),
                 num_tri, ptr(tri2vtx.contiguous()), num_vtx, ptr(vtx2xyz0.detach().contiguous()),
                 ptr(None if vtx2xyz1 is None else vtx2xyz1.detach().contiguous()), ptr(flags))
    return bvhnode2aabb


def make_bvhnode2aabb_from_bvhnodes(tri2vtx, vtx2xyz0, vtx2xyz1, bvhnodes, bvhnode2aabb):
    """Name of the reference's DLPack-level helper (TriMesh3/__init__.py:39-46)."""
    return update_bvhnode2aabb(tri2vtx, vtx2xyz0, bvhnodes, bvhnode2aabb, vtx2xyz1)


def self_intersection(tri2vtx: torch.Tensor, vtx2xyz: torch.Tensor, bvhnodes: torch.Tensor,
                      bvhnode2aabb: torch.Tensor, capacity: int = 1 << 16):
    """Self-intersecting triangle pairs through the BVH (the GPU form of
    ``del_msh_cpu::trimesh3_intersection::search_with_bvh_inside_branch``, as
    returned by del-msh-numpy's mesh_intersection binding): (edge2node2xyz
    (k, 2, 3) float32 segments, edge2tri (k, 2) uint32 triangle pairs), in no
    particular order.  Grows its buffer and repeats when more pairs exist."""
    num_tri, num_vtx = tri2vtx.shape[0], vtx2xyz.shape[0]
    device = tri2vtx.device
    assert_shape_dtype_device(tri2vtx, (num_tri, 3), torch.uint32, device)
    assert_shape_dtype_device(vtx2xyz, (num_vtx, 3), torch.float32, device)
    assert_shape_dtype_device(bvhnodes, (2 * num_tri - 1, 3), torch.uint32, device)
    assert_shape_dtype_device(bvhnode2aabb, (2 * num_tri - 1, 6), torch.float32, device)
    require_cuda(device)
    count = torch.zeros((1,), dtype=torch.int32, device=device)
    while True:
        pairs = torch.empty((capacity, 2), dtype=torch.uint32, device=device)
        segs = torch.empty((capacity, 2, 3), dtype=torch.float32, device=device)
        _native.call("dm_trimesh3_self_intersection", stream_ptr(device), num_tri, ptr(tri2vtx.contiguous()),
                     num_vtx, ptr(vtx2xyz.detach().contiguous()), ptr(bvhnodes.contiguous()),
                     ptr(bvhnode2aabb.contiguous()), capacity, ptr(pairs), ptr(segs), ptr(count))
        n = int(count.item())
        if n <= capacity:
            return segs[:n], pairs[:n]
        capacity = n
