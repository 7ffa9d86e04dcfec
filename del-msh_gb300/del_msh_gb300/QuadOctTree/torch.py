"""Quad/oct-trees from sorted unique Morton codes, on CUDA tensors.

Mirrors ``del_msh_dlpack/QuadOctTree/torch.py``: the binary radix tree with
per-branch depth (the LBVH's Karras construction), the branch -> octree-node
map, and the quad/oct-tree with cell centres and depths
(``del-msh-cpu/src/quad_oct_tree.rs``).
"""
from __future__ import annotations

import torch

from .. import _native
from ..util_torch import ptr, require_cuda, stream_ptr


def bnodes_and_bnode2depth_and_bnode2onode_and_idx2bnode(idx2morton: torch.Tensor, num_dim, max_depth=None):
    if max_depth is None:
        max_depth = 32 // num_dim
    num_idx = idx2morton.shape[0]
    num_bnode = num_idx - 1
    device = idx2morton.device
    assert idx2morton.dtype == torch.uint32
    require_cuda(device)
    bnodes = torch.empty((num_bnode, 3), device=device, dtype=torch.uint32)
    bnode2depth = torch.empty((num_bnode,), device=device, dtype=torch.uint32)
    bnode2onode = torch.empty((num_bnode,), device=device, dtype=torch.uint32)
    idx2bnode = torch.full((num_idx,), 2 ** 32 - 1, device=device, dtype=torch.uint32)
    scratch = torch.empty((_native.load().dm_quad_oct_tree_scratch_bytes(num_idx),), dtype=torch.uint8, device=device)
    _native.call("dm_quad_oct_tree_bnodes_and_bnode2depth_and_bnode2onode_and_idx2bnode", stream_ptr(device),
                 num_idx, ptr(idx2morton.contiguous()), num_dim, max_depth, ptr(bnodes), ptr(bnode2depth),
                 ptr(bnode2onode), ptr(idx2bnode), ptr(scratch), scratch.numel())
    return bnodes, bnode2depth, bnode2onode, idx2bnode


def make_tree_from_binary_radix_tree(bnodes, bnode2onode, bnode2depth, idx2bnode, idx2morton, num_dim: int,
                                     max_depth=None):
    num_bnode = bnodes.shape[0]
    num_idx = num_bnode + 1
    if max_depth is None:
        max_depth = 32 // num_dim
    nlink = 1 + 2 ** num_dim
    num_onode = int(bnode2onode[-1].item()) + 1  # one host read, as the reference wrapper
    device = bnodes.device
    require_cuda(device)
    onodes = torch.full((num_onode, nlink), 2 ** 32 - 1, device=device, dtype=torch.uint32)
    onode2depth = torch.zeros((num_onode,), device=device, dtype=torch.uint32)
    onode2center = torch.empty((num_onode, num_dim), device=device, dtype=torch.float32)
    idx2onode = torch.empty((num_idx,), device=device, dtype=torch.uint32)
    idx2center = torch.empty((num_idx, num_dim), device=device, dtype=torch.float32)
    _native.call("dm_quad_oct_tree_make_tree_from_binary_radix_tree", stream_ptr(device), num_idx,
                 ptr(bnodes.contiguous()), ptr(bnode2onode.contiguous()), ptr(bnode2depth.contiguous()),
                 ptr(idx2bnode.contiguous()), ptr(idx2morton.contiguous()), num_dim, max_depth, num_onode,
                 ptr(onodes), ptr(onode2depth), ptr(onode2center), ptr(idx2onode), ptr(idx2center))
    return onodes, onode2depth, onode2center, idx2onode, idx2center


def aggregate(idx2val: torch.Tensor, idx2onode: torch.Tensor, onodes: torch.Tensor) -> torch.Tensor:
    """Sum of idx2val over the leaves below each octree node (atomic adds)."""
    num_idx, num_vdim = idx2val.shape
    num_onode, num_link = onodes.shape
    device = idx2val.device
    require_cuda(device)
    out = torch.empty((num_onode, num_vdim), device=device, dtype=torch.float32)
    _native.call("dm_quad_oct_tree_aggregate", stream_ptr(device), num_idx, num_vdim, ptr(idx2val.contiguous()),
                 ptr(idx2onode.contiguous()), num_link, ptr(onodes.contiguous()), num_onode, ptr(out))
    return out


class QuadOctTree:
    def __init__(self):
        pass

    def construct_from_idx2morton(self, idx2morton: torch.Tensor, num_dim: int, is_save_intermediate=False):
        self.num_dim = num_dim
        bnodes, bnode2depth, bnode2onode, idx2bnode = bnodes_and_bnode2depth_and_bnode2onode_and_idx2bnode(
            idx2morton, num_dim)
        (self.onodes, self.onode2depth, self.onode2center, self.idx2onode,
         self.idx2center) = make_tree_from_binary_radix_tree(bnodes, bnode2onode, bnode2depth, idx2bnode, idx2morton,
                                                             num_dim)
        if is_save_intermediate:
            self.bnodes = bnodes
            self.bnode2depth = bnode2depth
            self.bnode2onode = bnode2onode
            self.idx2bnode = idx2bnode

    def aggregate(self, idx2val: torch.Tensor) -> torch.Tensor:
        return aggregate(idx2val, self.idx2onode, self.onodes)
