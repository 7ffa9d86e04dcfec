"""The allocation-free refit entry point, called through the C ABI.

dm_bvhnode2aabb_update_aabb_noalloc serves callers that cannot allocate
device memory (a per-frame refit under a no-allocation rule, a plugin whose
host owns the CUDA allocator, an FFI caller with only its own arrays): its
scratch is a static device array inside the library.  Its result must equal
the allocating entry point's, call after call, since the shared array keeps
the previous call's contents.  This file sorts last so that a run stopping at
the first failure has already run every other test.
"""
import numpy as np
import pytest

from helpers import bits, to_dev, to_np

from del_msh_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _refit(torch, noalloc, tri, vtx, bvh, num_tri, vtx1=None):
    from del_msh_gb300 import _native
    aabb = torch.full((2 * num_tri - 1, 6), float("nan"), dtype=torch.float32, device="cuda:0")
    sp = torch.cuda.current_stream().cuda_stream
    v1 = None if vtx1 is None else vtx1.data_ptr()
    if noalloc:
        _native.call("dm_bvhnode2aabb_update_aabb_noalloc", sp, 2 * num_tri - 1, aabb.data_ptr(), bvh.data_ptr(),
                     num_tri, tri.data_ptr(), vtx.shape[0], vtx.data_ptr(), v1)
    else:
        _native.call("dm_bvhnode2aabb_update_aabb", sp, 2 * num_tri - 1, aabb.data_ptr(), 0, bvh.data_ptr(),
                     num_tri, tri.data_ptr(), vtx.shape[0], vtx.data_ptr(), v1, None)
    return to_np(aabb, torch)


def test_noalloc_refit_matches_allocating_refit(cuda, oracle):
    """Two deformed frames in a row, then a frame whose boxes also enclose a
    second vertex array: the allocation-free refit equals the allocating
    entry point and the oracle (del-msh-cpu's refit restated), bit for bit."""
    torch = cuda
    from del_msh_gb300.TriMesh3 import torch as TriMesh3
    tri, vtx = W.displaced_torus(160, seed=21)
    T = tri.shape[0]
    d_tri = to_dev(tri, torch)
    bvh, _ = TriMesh3.make_bvhnodes_bvhnode2aabb(d_tri, to_dev(vtx, torch))
    bvh_np = to_np(bvh, torch)
    phase = np.random.default_rng(21).uniform(0, 6.28, vtx.shape[0])
    frames = [(vtx + 0.01 * np.sin(phase + f)[:, None]).astype(np.float32) for f in range(3)]
    for frame in range(3):  # calls in a row share the static flags
        v0 = frames[frame]
        v1 = frames[0] * np.float32(1.02) if frame == 2 else None  # the two-position union
        d0, d1 = to_dev(v0, torch), (None if v1 is None else to_dev(v1, torch))
        want = _refit(torch, False, d_tri, d0, bvh, T, d1)
        got = _refit(torch, True, d_tri, d0, bvh, T, d1)
        assert np.array_equal(bits(got), bits(want)), f"frame {frame}"
        assert np.array_equal(bits(got), bits(oracle.bvhnode2aabb(bvh_np, tri, v0, v1))), f"frame {frame}"
    from del_msh_gb300 import _native
    assert _native.device_status(clear=True) == 0


def test_noalloc_refit_allocates_nothing(cuda):
    """After a first call (which looks up the static array's address), a call
    changes neither torch's allocations nor the device's free memory."""
    torch = cuda
    from del_msh_gb300.TriMesh3 import torch as TriMesh3
    tri, vtx = W.displaced_torus(64, seed=22)
    T = tri.shape[0]
    d_tri, d_vtx = to_dev(tri, torch), to_dev(vtx, torch)
    bvh, _ = TriMesh3.make_bvhnodes_bvhnode2aabb(d_tri, d_vtx)
    aabb = torch.empty((2 * T - 1, 6), dtype=torch.float32, device="cuda:0")
    from del_msh_gb300 import _native
    sp = torch.cuda.current_stream().cuda_stream

    def call():
        _native.call("dm_bvhnode2aabb_update_aabb_noalloc", sp, 2 * T - 1, aabb.data_ptr(), bvh.data_ptr(), T,
                     d_tri.data_ptr(), vtx.shape[0], d_vtx.data_ptr(), None)

    call()
    torch.cuda.synchronize()
    alloc0, free0 = torch.cuda.memory_allocated(), torch.cuda.mem_get_info()[0]
    call()
    torch.cuda.synchronize()
    assert torch.cuda.memory_allocated() == alloc0
    assert torch.cuda.mem_get_info()[0] == free0
    assert _native.device_status(clear=True) == 0


def test_noalloc_rejects_meshes_beyond_its_maximum(cuda):
    from del_msh_gb300 import _native
    with pytest.raises(_native.DelMshError, match="4194305"):
        _native.call("dm_bvhnode2aabb_update_aabb_noalloc", 0, 2 * 4_194_306 - 1, 1, 1, 4_194_306, 1, 1, 1, None)
