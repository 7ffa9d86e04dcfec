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


def _refit(torch, noalloc, tri, vtx, bvh, num_tri):
    from del_msh_gb300 import _native
    aabb = torch.full((2 * num_tri - 1, 6), float("nan"), dtype=torch.float32, device="cuda:0")
    sp = torch.cuda.current_stream().cuda_stream
    if noalloc:
        _native.call("dm_bvhnode2aabb_update_aabb_noalloc", sp, 2 * num_tri - 1, aabb.data_ptr(), bvh.data_ptr(),
                     num_tri, tri.data_ptr(), vtx.shape[0], vtx.data_ptr(), None)
    else:
        _native.call("dm_bvhnode2aabb_update_aabb", sp, 2 * num_tri - 1, aabb.data_ptr(), 0, bvh.data_ptr(),
                     num_tri, tri.data_ptr(), vtx.shape[0], vtx.data_ptr(), None, None)
    return to_np(aabb, torch)


def test_noalloc_refit_matches_allocating_refit(cuda):
    torch = cuda
    from del_msh_gb300.TriMesh3 import torch as TriMesh3
    tri, vtx = W.displaced_torus(160, seed=21)
    T = tri.shape[0]
    d_tri = to_dev(tri, torch)
    bvh, _ = TriMesh3.make_bvhnodes_bvhnode2aabb(d_tri, to_dev(vtx, torch))
    phase = np.random.default_rng(21).uniform(0, 6.28, vtx.shape[0])
    for frame in range(2):  # two calls in a row share the static flags
        v = to_dev((vtx + 0.01 * np.sin(phase + frame)[:, None]).astype(np.float32), torch)
        want = _refit(torch, False, d_tri, v, bvh, T)
        got = _refit(torch, True, d_tri, v, bvh, T)
        assert np.array_equal(bits(got), bits(want)), f"frame {frame}"
    from del_msh_gb300 import _native
    assert _native.device_status(clear=True) == 0


def test_noalloc_rejects_meshes_beyond_its_maximum(cuda):
    from del_msh_gb300 import _native
    with pytest.raises(_native.DelMshError, match="4194305"):
        _native.call("dm_bvhnode2aabb_update_aabb_noalloc", 0, 2 * 4_194_306 - 1, 1, 1, 4_194_306, 1, 1, 1, None)
