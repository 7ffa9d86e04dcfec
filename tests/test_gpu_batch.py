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


def _soup(n, seed):
    return W.clustered_soup(n, num_cluster=4, seed=seed)


def _torus(nmajor, nminor, seed):
    tri, vtx = W.torus_zup(1.0, 0.35, nmajor, nminor)
    rng = np.random.default_rng(seed)
    return tri, (vtx.astype(np.float64) + rng.uniform(-0.01, 0.01, vtx.shape)).astype(np.float32)


def _check_trees(torch, oracle, b, meshes):
    for m, (tri, vtx) in enumerate(meshes):
        bvh, aabb = b.mesh_tree(m)
        ref = oracle.build(tri, vtx)
        assert np.array_equal(to_np(bvh, torch), ref["bvhnodes"]), m
        assert np.array_equal(bits(to_np(aabb, torch)), bits(ref["bvhnode2aabb"])), m


@pytest.mark.parametrize("sizes", [
    # largest mesh in (16384, 32768]: clusters of two blocks
    "pairs",
    # largest mesh in (32768, 65536]: clusters of four blocks
    "quads",
    # largest mesh above 65536: the global (mesh, code) sort
    "global",
])
def test_batch_build_large_meshes_match_oracle(cuda, oracle, sizes):
    """Meshes at and around the block (16384) and cluster capacities, clustered
    soups whose runs of equal codes cross block boundaries, and small meshes
    built by single blocks in the same launch."""
    torch = cuda
    from del_msh_gb300 import _native
    from del_msh_gb300.batch import MeshBatch
    meshes = [W.icosphere(1), _soup(700, 1), _soup(16384, 2), _soup(16385, 3), _torus(128, 64, 4)]
    if sizes == "pairs":
        meshes += [_soup(32768, 5), _torus(128, 128, 6), _soup(20000, 7)]
    elif sizes == "quads":
        meshes += [_soup(32769, 8), _torus(256, 128, 9), _soup(65536, 10), _soup(50001, 11)]
    else:
        meshes += [_soup(70000, 12), _torus(256, 128, 13)]
    meshes.append((np.array([[0, 1, 2]], np.uint32), np.array([[0, 0, 0], [1, 0, 0], [0, 1, 1]], np.float32)))
    b = MeshBatch(meshes)
    b.build()
    torch.cuda.synchronize()
    _check_trees(torch, oracle, b, meshes)
    assert _native.device_status(clear=True) == 0


def test_batch_build_understated_max_tri(cuda, oracle):
    """A mesh above the max_tri_per_mesh the call was given raises status bit 4
    and gets the documented placeholder tree (branch i: leaf i, branch i + 1),
    with the boxes of that tree; the other meshes are unaffected."""
    torch = cuda
    from del_msh_gb300 import _native
    from del_msh_gb300.batch import MeshBatch
    meshes = [_soup(3000, 1), _soup(9000, 2), W.icosphere(2)]
    b = MeshBatch(meshes)
    b.max_tri = 5000  # understated: mesh 1 has 9000 triangles
    _native.device_status(clear=True)
    b.build()
    torch.cuda.synchronize()
    assert _native.device_status(clear=True) == 4
    for m in (0, 2):
        tri, vtx = meshes[m]
        bvh, aabb = b.mesh_tree(m)
        ref = oracle.build(tri, vtx)
        assert np.array_equal(to_np(bvh, torch), ref["bvhnodes"]), m
        assert np.array_equal(bits(to_np(aabb, torch)), bits(ref["bvhnode2aabb"])), m
    T = 9000
    bvh, aabb = b.mesh_tree(1)
    bvh, aabb = to_np(bvh, torch).astype(np.int64), to_np(aabb, torch)
    nb = T - 1
    i = np.arange(nb)
    assert np.array_equal(bvh[:nb, 0], np.where(i == 0, 0xFFFFFFFF, i - 1))
    assert np.array_equal(bvh[:nb, 1], nb + i)
    assert np.array_equal(bvh[:nb, 2], np.where(i + 1 < nb, i + 1, nb + i + 1))
    j = np.arange(T)
    assert np.array_equal(bvh[nb:, 0], np.minimum(j, nb - 1))
    assert np.array_equal(bvh[nb:, 1], j)
    assert (bvh[nb:, 2] == 0xFFFFFFFF).all()
    # the root box is the box of every triangle, whatever the tree
    root = oracle.build(*meshes[1])["bvhnode2aabb"][0]
    assert np.array_equal(bits(aabb[0]), bits(root))


def test_full_ragged_batch_4096(cuda, oracle):
    """The full ragged batch: 4096 meshes (37.9M triangles, counts realised up
    to 65024, so clusters of four blocks), each with its 64x64 orthographic
    image.  Every mesh's tree, boxes and image equal the oracle's bit for bit."""
    torch = cuda
    from del_msh_gb300 import _native
    from del_msh_gb300.batch import MeshBatch, ortho_transforms
    meshes = W.ragged_batch(num_mesh=4096, tmin=64, tmax=65536, seed=0)
    b = MeshBatch(meshes)
    assert b.max_tri > 49152 and b.total_tri > 37_000_000
    tf = ortho_transforms(meshes)
    b.build()
    b.alloc_cast(64, 64)
    p2t, tt = b.cast_pixels(torch.from_numpy(tf).to("cuda:0"))
    torch.cuda.synchronize()
    bvh_all, aabb_all = to_np(b.bvhnodes, torch), bits(to_np(b.bvhnode2aabb, torch))
    p2t, tt = to_np(p2t, torch), bits(to_np(tt, torch))
    for m, (tri, vtx) in enumerate(meshes):
        ref = oracle.build(tri, vtx)
        a = int(b.node_off[m])
        n = 2 * tri.shape[0] - 1
        assert np.array_equal(bvh_all[a:a + n], ref["bvhnodes"]), m
        assert np.array_equal(aabb_all[a:a + n], bits(ref["bvhnode2aabb"])), m
        r_p2t, r_tt = oracle.pix2tri(tri, vtx, ref["bvhnodes"], ref["bvhnode2aabb"], tf[m], 64, 64)
        assert np.array_equal(p2t[m], r_p2t), m
        assert np.array_equal(tt[m], bits(r_tt)), m
    assert _native.device_status(clear=True) == 0


def test_batch_cast_through_warp_tier(cuda, oracle):
    """The batched cast with a one-entry step budget: rays of the soups that
    reach long runs of chain links go through the warp tier (BatchJob), and
    every image still equals the oracle's bit for bit."""
    torch = cuda
    from del_msh_gb300 import _native
    from del_msh_gb300.batch import MeshBatch, ortho_transforms
    meshes = [W.clustered_soup(8_000, num_cluster=2, seed=6), _torus(64, 32, 7),
              W.clustered_soup(20_000, num_cluster=3, seed=8), W.icosphere(2)]
    b = MeshBatch(meshes)
    b.build()
    tf = ortho_transforms(meshes)
    b.alloc_cast(48, 40)
    before = _native.get_tuning()
    try:
        _native.set_tuning(**dict(before, cast_long_steps=1))
        p2t, tt = b.cast_pixels(torch.from_numpy(tf).to("cuda:0"))
        torch.cuda.synchronize()
    finally:
        _native.set_tuning(**before)
    p2t, tt = to_np(p2t, torch), bits(to_np(tt, torch))
    hits = 0
    for m, (tri, vtx) in enumerate(meshes):
        ref = oracle.build(tri, vtx)
        r_p2t, r_tt = oracle.pix2tri(tri, vtx, ref["bvhnodes"], ref["bvhnode2aabb"], tf[m], 48, 40)
        assert np.array_equal(p2t[m], r_p2t), m
        assert np.array_equal(tt[m], bits(r_tt)), m
        hits += int((r_p2t != 0xFFFFFFFF).sum())
    assert hits > 1000
    assert _native.device_status(clear=True) == 0


def test_mesh_id_partition_matches_whole_batch(cuda):
    """Meshes split by id over 3 ranks (each rank's MeshBatch built and cast
    one after another on this GPU): every mesh's tree, boxes and image equal
    the whole batch's, bit for bit."""
    torch = cuda
    from del_msh_gb300 import _native
    from del_msh_gb300 import partition as P
    from del_msh_gb300.batch import MeshBatch, ortho_transforms
    meshes = W.ragged_batch(num_mesh=60, tmin=64, tmax=40000, seed=21)
    whole = MeshBatch(meshes)
    whole.build()
    whole.alloc_cast(32, 24)
    whole.cast_pixels(torch.from_numpy(ortho_transforms(meshes)).to("cuda:0"))
    parts = P.partition_meshes([t.shape[0] for t, _ in meshes], 3)
    results = []
    for ids in parts:
        sub = [meshes[m] for m in ids]
        b = MeshBatch(sub)
        b.build()
        b.alloc_cast(32, 24)
        p2t, tt = b.cast_pixels(torch.from_numpy(ortho_transforms(sub)).to("cuda:0"))
        outs = []
        for k in range(len(ids)):
            bvh, aabb = b.mesh_tree(k)
            outs.append((to_np(bvh, torch), bits(to_np(aabb, torch)), to_np(p2t[k], torch), bits(to_np(tt[k], torch))))
        results.append((ids, outs))
    got = P.gather_meshes(results, len(meshes))
    for m in range(len(meshes)):
        bvh, aabb = whole.mesh_tree(m)
        want = (to_np(bvh, torch), bits(to_np(aabb, torch)), to_np(whole.pix2tri[m], torch),
                bits(to_np(whole.pix2t[m], torch)))
        for a, w in zip(got[m], want):
            assert np.array_equal(a, w), m
    assert _native.device_status(clear=True) == 0
