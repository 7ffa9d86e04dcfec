"""Package-root form of the TriMesh3 BVH helper of
del_msh_dlpack/TriMesh3/__init__.py (make_bvhnode2aabb_from_bvhnodes):
caller-allocated arrays, results in place, launched on ``stream_ptr`` (0 =
the default stream).  Arrays are torch CUDA tensors or objects
torch.from_dlpack accepts.  The torch front-end is in ``.torch``."""
from __future__ import annotations

from .._root import as_tensor, call_on_stream


def make_bvhnode2aabb_from_bvhnodes(tri2vtx, vtx2xyz0, vtx2xyz1, bvhnodes, bvhnode2aabb, stream_ptr=0):
    """Every node's AABB of the tree bvhnodes for the vertices vtx2xyz0
    (enclosing vtx2xyz1 too when it is given with the same vertex count).
    Replaces bvhnode2aabb_update_aabb (del-msh-dlpack/src/bvhnode2aabb.rs:15-108)."""
    from .. import _native
    tri2vtx, vtx2xyz0, bvhnodes, bvhnode2aabb = map(as_tensor, (tri2vtx, vtx2xyz0, bvhnodes, bvhnode2aabb))
    v1 = None if vtx2xyz1 is None else as_tensor(vtx2xyz1)
    if v1 is not None and v1.shape[0] != vtx2xyz0.shape[0]:
        v1 = None  # the binding ignores a second position array of another size
    num_tri = tri2vtx.shape[0]
    call_on_stream(stream_ptr, tri2vtx.device, 0, lambda _: _native.call(
        "dm_bvhnode2aabb_update_aabb", stream_ptr, bvhnodes.shape[0], bvhnode2aabb.data_ptr(), 0,
        bvhnodes.data_ptr(), num_tri, tri2vtx.data_ptr(), vtx2xyz0.shape[0], vtx2xyz0.data_ptr(),
        None if v1 is None else v1.data_ptr(), None))
