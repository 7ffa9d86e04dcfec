"""Batched build + cast of ragged meshes: every mesh's slice equals the
single-mesh path and the oracle bit for bit, eagerly and replayed from a CUDA
graph."""
import numpy as np
import pytest

from helpers import bits, to_np

from del_msh_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _meshes():
    ms = W.ragged_batch(num_mesh=40, tmin=64, tmax=6000, seed=3)
    ms.append((np.array([[0, 1, 2]], np.uint32), np.array([[0, 0, 0], [1, 0, 0], [0, 1, 1]], np.float32)))  # T = 1
    ms.append(W.icosphere(0))  # T = 20
    ms.append((np.array([[0, 1, 2], [2, 1, 0]], np.uint32), np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)))
    ms.append(W.clustered_soup(5000, num_cluster=3, seed=5))  # duplicate Morton codes
    return ms


@pytest.mark.parametrize("want_heights", [False, True])
def test_batch_build_and_cast_match_single_and_oracle(cuda, oracle, want_heights):
    torch = cuda
    from del_msh_gb300.batch import MeshBatch, PlainPath, ortho_transforms
    meshes = _meshes()
    b = MeshBatch(meshes, want_heights=want_heights)
    b.build()
    tf = torch.from_numpy(ortho_transforms(meshes)).to("cuda:0")
    b.alloc_cast(24, 20)
    p2t, tt = b.cast_pixels(tf)
    plain = PlainPath(b)
    plain.build()
    plain.alloc_cast(24, 20)
    q2t, qt = plain.cast_pixels(tf)
    torch.cuda.synchronize()
    p2t, tt, q2t, qt = to_np(p2t, torch), to_np(tt, torch), to_np(q2t, torch), to_np(qt, torch)
    heights = to_np(b.heights, torch) if want_heights else None
    for m, (tri, vtx) in enumerate(meshes):
        bvh, aabb = b.mesh_tree(m)
        ref = oracle.build(tri, vtx)
        assert np.array_equal(to_np(bvh, torch), ref["bvhnodes"]), m
        assert np.array_equal(bits(to_np(aabb, torch)), bits(ref["bvhnode2aabb"])), m
        assert np.array_equal(to_np(plain.trees[m][0], torch), ref["bvhnodes"]), m
        assert np.array_equal(bits(to_np(plain.trees[m][1], torch)), bits(ref["bvhnode2aabb"])), m
        if want_heights:
            assert heights[m] == oracle.tree_height(ref["bvhnodes"], tri.shape[0]), m
        r_p2t, r_tt = oracle.pix2tri(tri, vtx, ref["bvhnodes"], ref["bvhnode2aabb"], ortho_transforms([meshes[m]])[0],
                                     24, 20)
        assert np.array_equal(p2t[m], r_p2t), m
        assert np.array_equal(bits(tt[m]), bits(r_tt)), m
    assert np.array_equal(p2t, q2t)
    assert np.array_equal(bits(tt), bits(qt))
    from del_msh_gb300 import _native
    assert _native.device_status(clear=True) == 0


def test_batch_graph_replay_follows_vertex_updates(cuda, oracle):
    torch = cuda
    from del_msh_gb300.batch import MeshBatch, ortho_transforms
    meshes = _meshes()
    b = MeshBatch(meshes)
    tf = torch.from_numpy(ortho_transforms(meshes, margin=0.3)).to("cuda:0")
    b.alloc_cast(16, 16)
    b.capture(tf)
    rng = np.random.default_rng(0)
    for frame in range(2):
        new = [(t, (v + rng.uniform(-0.01, 0.01, v.shape)).astype(np.float32)) for t, v in meshes]
        b.vtx2xyz.copy_(torch.from_numpy(np.concatenate([v for _, v in new])))
        b.replay()
        torch.cuda.synchronize()
        got = to_np(b.pix2tri, torch)
        for m, (tri, vtx) in enumerate(new):
            ref = oracle.build(tri, vtx)
            bvh, aabb = b.mesh_tree(m)
            assert np.array_equal(to_np(bvh, torch), ref["bvhnodes"]), (frame, m)
            r_p2t, _ = oracle.pix2tri(tri, vtx, ref["bvhnodes"], ref["bvhnode2aabb"],
                                      ortho_transforms([meshes[m]], margin=0.3)[0], 16, 16)
            assert np.array_equal(got[m], r_p2t), (frame, m)
