"""Launch-parameter tuning: the host-side table (CPU) and result identity of
every compiled choice against the oracle (GPU)."""
import numpy as np
import pytest

from helpers import bits, to_dev, to_np

from del_msh_gb300 import workloads as W


def test_tuning_roundtrip_and_validation():
    from del_msh_gb300 import _native
    from del_msh_gb300.autotune import CAST_CHOICES, DEFAULT, PHASE_CHOICES, SORT_WINDOWS, TILE_CHOICES
    before = _native.get_tuning()
    try:
        for threads, frames in CAST_CHOICES:
            for tile_w in TILE_CHOICES:
                for window in SORT_WINDOWS:
                    _native.set_tuning(threads, frames, tile_w, window)  # phase minima 0: the default, 6
                    assert _native.get_tuning() == dict(cast_threads=threads, cast_stack=frames, tile_w=tile_w,
                                                        sort_window=window, cast_refill_min=6, cast_leaf_min=6,
                                                        cast_ascend_min=6, cast_long_steps=64, batch_path=0,
                                                        batch_cluster=0)
        for mins in PHASE_CHOICES + [(1, 32, 32), (32, 1, 32), (32, 32, 1)]:
            _native.set_tuning(128, 64, 8, 4, *mins)
            assert tuple(_native.get_tuning()[k] for k in ("cast_refill_min", "cast_leaf_min",
                                                           "cast_ascend_min")) == mins
        _native.set_tuning(**DEFAULT)
        for bad in [(96, 64, 8, 4), (128, 48, 8, 4), (128, 64, 3, 4), (128, 64, 64, 4), (128, 64, 8, 5),
                    (128, 64, 8, 4, 33, 6, 6), (128, 64, 8, 4, 6, 40, 6), (128, 64, 8, 4, 6, 6, 33),
                    (128, 64, 8, 4, 6, 6, 6, (1 << 30) + 1), (128, 64, 8, 4, 6, 6, 6, 64, 2),
                    (128, 64, 8, 4, 6, 6, 6, 64, 0, 3)]:
            with pytest.raises(_native.DelMshError):
                _native.set_tuning(*bad)
            assert _native.get_tuning() == DEFAULT  # a rejected choice changes nothing
    finally:
        _native.set_tuning(**before)


def test_build_classes_roundtrip_and_validation():
    from del_msh_gb300 import _native
    before = _native.get_build_classes()
    try:
        good = [dict(max_tri=1 << 16, build_path=1, sort_radix=10, topo_threads=128),
                dict(max_tri=1 << 21, build_path=0, sort_radix=0, topo_threads=512),
                dict(max_tri=0xFFFFFFFF, build_path=1, sort_radix=8, topo_threads=256)]
        _native.set_build_classes(good)
        assert _native.get_build_classes() == good
        for bad in ([dict(max_tri=10), dict(max_tri=5)],  # bounds must ascend
                    [dict(max_tri=10, build_path=2)], [dict(max_tri=10, sort_radix=9)],
                    [dict(max_tri=10, topo_threads=64)], [dict(max_tri=k + 1) for k in range(9)]):
            with pytest.raises(_native.DelMshError):
                _native.set_build_classes(bad)
            assert _native.get_build_classes() == good  # a rejected table changes nothing
        _native.set_build_classes([])
        assert _native.get_build_classes() == []
    finally:
        _native.set_build_classes(before)


def test_apply_ignores_foreign_table(tmp_path):
    import json
    from del_msh_gb300 import _native, autotune
    before = _native.get_tuning()
    p = tmp_path / "t.json"
    p.write_text(json.dumps({"device": "not this GPU", "best": dict(cast_threads=64, cast_stack=64, tile_w=4,
                                                                        sort_window=8)}))
    assert autotune.apply(p) is None
    assert _native.get_tuning() == before


@pytest.mark.gpu
def test_every_tuning_choice_matches_oracle(cuda, oracle):
    torch = cuda
    from del_msh_gb300 import _native
    from del_msh_gb300.autotune import CAST_CHOICES, PHASE_CHOICES, SORT_WINDOWS, TILE_CHOICES
    from del_msh_gb300.Pix2Tri import torch as Pix2Tri
    from del_msh_gb300.TriMesh3 import torch as TriMesh3
    tri, vtx = W.displaced_torus(96, seed=11)
    ref = oracle.build(tri, vtx)
    m = W.pinhole_ndc2world(W.random_viewpoint(3.0, seed=2), aspect=200 / 150)
    r_p2t, r_tt = oracle.pix2tri(tri, vtx, ref["bvhnodes"], ref["bvhnode2aabb"], m, 200, 150)
    d_tri, d_vtx = to_dev(tri, torch), to_dev(vtx, torch)
    m_row = torch.from_numpy(np.ascontiguousarray(m.reshape(4, 4).T)).to("cuda:0")
    before = _native.get_tuning()
    try:
        for window in SORT_WINDOWS:
            _native.set_tuning(before["cast_threads"], before["cast_stack"], before["tile_w"], window)
            bvh, aabb = TriMesh3.make_bvhnodes_bvhnode2aabb(d_tri, d_vtx)
            assert np.array_equal(to_np(bvh, torch), ref["bvhnodes"]), window
            assert np.array_equal(bits(to_np(aabb, torch)), bits(ref["bvhnode2aabb"])), window
        for threads, frames in CAST_CHOICES:
            for tile_w in TILE_CHOICES:
                _native.set_tuning(threads, frames, tile_w, before["sort_window"])
                p2t, tt = Pix2Tri.by_raycasting(d_tri, d_vtx, bvh, aabb, m_row, (200, 150), return_depth=True)
                assert np.array_equal(to_np(p2t, torch), r_p2t), (threads, frames, tile_w)
                assert np.array_equal(bits(to_np(tt, torch)), bits(r_tt)), (threads, frames, tile_w)
        # results do not depend on when a warp runs each phase
        for mins in PHASE_CHOICES + [(1, 32, 32), (32, 1, 32), (32, 32, 1), (32, 32, 32)]:
            _native.set_tuning(before["cast_threads"], before["cast_stack"], before["tile_w"], before["sort_window"],
                               *mins)
            p2t, tt = Pix2Tri.by_raycasting(d_tri, d_vtx, bvh, aabb, m_row, (200, 150), return_depth=True)
            assert np.array_equal(to_np(p2t, torch), r_p2t), mins
            assert np.array_equal(bits(to_np(tt, torch)), bits(r_tt)), mins
    finally:
        _native.set_tuning(**before)
    assert _native.device_status(clear=True) == 0


@pytest.mark.gpu
@pytest.mark.parametrize("mesh", ["torus", "soup", "small"])
def test_every_build_choice_matches_oracle(cuda, oracle, mesh):
    """Every single-mesh build choice of the size classes (cooperative front
    or separate kernels, 8- or 10-bit digits, topology block size) builds the
    oracle's tree and boxes."""
    torch = cuda
    from del_msh_gb300 import _native
    from del_msh_gb300.autotune import BUILD_CHOICES
    from del_msh_gb300.TriMesh3 import torch as TriMesh3
    if mesh == "torus":
        tri, vtx = W.displaced_torus(400, seed=12)  # 320k triangles
    elif mesh == "soup":
        tri, vtx = W.clustered_soup(120_000, num_cluster=5, seed=13)
    else:
        tri, vtx = W.jittered_icosphere(2, seed=14)
    ref = oracle.build(tri, vtx)
    d_tri, d_vtx = to_dev(tri, torch), to_dev(vtx, torch)
    before = _native.get_build_classes()
    try:
        for c in BUILD_CHOICES:
            _native.set_build_classes([dict(max_tri=0xFFFFFFFF, **c)])
            bvh, aabb = TriMesh3.make_bvhnodes_bvhnode2aabb(d_tri, d_vtx)
            assert np.array_equal(to_np(bvh, torch), ref["bvhnodes"]), c
            assert np.array_equal(bits(to_np(aabb, torch)), bits(ref["bvhnode2aabb"])), c
    finally:
        _native.set_build_classes(before)
    assert _native.device_status(clear=True) == 0


@pytest.mark.gpu
def test_every_batch_choice_matches_oracle(cuda, oracle):
    """Every batched build choice (on chip with the fewest or more blocks per
    large mesh, or the global sort) builds every mesh's oracle tree and boxes."""
    torch = cuda
    from del_msh_gb300 import _native
    from del_msh_gb300.autotune import BATCH_CHOICES
    from del_msh_gb300.batch import MeshBatch
    meshes = W.ragged_batch(num_mesh=30, tmin=64, tmax=30000, seed=15)
    refs = [oracle.build(t, v) for t, v in meshes]
    b = MeshBatch(meshes)
    before = _native.get_tuning()
    try:
        for c in BATCH_CHOICES:
            _native.set_tuning(**dict(before, **c))
            b.build()
            for m, r in enumerate(refs):
                bvh, aabb = b.mesh_tree(m)
                assert np.array_equal(to_np(bvh, torch), r["bvhnodes"]), (c, m)
                assert np.array_equal(bits(to_np(aabb, torch)), bits(r["bvhnode2aabb"])), (c, m)
    finally:
        _native.set_tuning(**before)
    assert _native.device_status(clear=True) == 0


@pytest.mark.gpu
def test_shallow_stack_overflows_to_deeper_tiers(cuda, oracle):
    """The 32-frame on-chip stack on the duplicate-heavy soup: rays that need
    more go through the overflow tiers and still give the oracle's hits."""
    torch = cuda
    from del_msh_gb300 import _native
    from del_msh_gb300.SearchBvh3 import torch as SearchBvh3
    from del_msh_gb300.TriMesh3 import torch as TriMesh3
    tri, vtx = W.clustered_soup(60_000, seed=9)
    org, d = W.cube_boundary_rays(20_000, seed=9)
    ref = oracle.build(tri, vtx)
    r_hit, r_t = oracle.cast_rays(org, d, tri, vtx, ref["bvhnodes"], ref["bvhnode2aabb"])
    before = _native.get_tuning()
    try:
        _native.set_tuning(128, 32, before["tile_w"], before["sort_window"])
        d_tri, d_vtx = to_dev(tri, torch), to_dev(vtx, torch)
        bvh, aabb = TriMesh3.make_bvhnodes_bvhnode2aabb(d_tri, d_vtx)
        hit, t = SearchBvh3.first_intersection_ray(to_dev(org, torch), to_dev(d, torch), d_tri, d_vtx, bvh, aabb)
        assert np.array_equal(to_np(hit, torch), r_hit)
        assert np.array_equal(bits(to_np(t, torch)), bits(r_t))
    finally:
        _native.set_tuning(**before)
    assert _native.device_status(clear=True) == 0


@pytest.mark.gpu
@pytest.mark.parametrize("long_steps", [1, 16])
def test_warp_tier_matches_oracle(cuda, oracle, long_steps):
    """With a tiny step budget the persistent cast hands every ray that
    reaches a long run of chain links (once its warp has no more rays to
    take) to the warp tier, which folds the links 32 at a time; on a soup with
    rays aimed at its clusters (runs of equal codes) hundreds of rays go
    there, and the hits equal the oracle's bit for bit.  A smooth mesh, with
    no long chains, keeps the oracle's bits under the same budget."""
    torch = cuda
    from del_msh_gb300 import _native
    from del_msh_gb300.Pix2Tri import torch as Pix2Tri
    from del_msh_gb300.TriMesh3 import torch as TriMesh3
    tri, vtx = W.displaced_torus(96, seed=11)
    ref = oracle.build(tri, vtx)
    m = W.pinhole_ndc2world(W.random_viewpoint(3.0, seed=2), aspect=120 / 90)
    r_p2t, r_tt = oracle.pix2tri(tri, vtx, ref["bvhnodes"], ref["bvhnode2aabb"], m, 120, 90)
    stri, svtx = W.clustered_soup(200_000, num_cluster=4, seed=9)
    # rays from the cube boundary aimed at triangles, so that they cross the
    # clusters' runs of equal codes (the tree's long chains)
    org, _ = W.cube_boundary_rays(4_000, seed=9)
    rng = np.random.default_rng(9)
    target = svtx[stri[rng.integers(0, stri.shape[0], org.shape[0])]].mean(axis=1)
    target = target + rng.uniform(-2e-4, 2e-4, target.shape)
    d = (target - org).astype(np.float32)
    sref = oracle.build(stri, svtx)
    r_hit, r_t = oracle.cast_rays(org, d, stri, svtx, sref["bvhnodes"], sref["bvhnode2aabb"])
    assert (r_hit != 0xFFFFFFFF).sum() > 1000
    L = _native.load()
    before = _native.get_tuning()
    try:
        _native.set_tuning(**dict(before, cast_long_steps=long_steps))
        d_tri, d_vtx = to_dev(tri, torch), to_dev(vtx, torch)
        bvh, aabb = TriMesh3.make_bvhnodes_bvhnode2aabb(d_tri, d_vtx)
        m_row = torch.from_numpy(np.ascontiguousarray(m.reshape(4, 4).T)).to("cuda:0")
        p2t, tt = Pix2Tri.by_raycasting(d_tri, d_vtx, bvh, aabb, m_row, (120, 90), return_depth=True)
        assert np.array_equal(to_np(p2t, torch), r_p2t)
        assert np.array_equal(bits(to_np(tt, torch)), bits(r_tt))
        s_tri, s_vtx = to_dev(stri, torch), to_dev(svtx, torch)
        sbvh, saabb = TriMesh3.make_bvhnodes_bvhnode2aabb(s_tri, s_vtx)
        n, T, V = org.shape[0], stri.shape[0], svtx.shape[0]
        hit = torch.empty((n,), dtype=torch.int32, device="cuda:0")
        t = torch.empty((n,), dtype=torch.float32, device="cuda:0")
        cs = L.dm_cast_scratch_bytes(n, T)
        scr = torch.empty((cs,), dtype=torch.uint8, device="cuda:0")
        o_dev, d_dev = to_dev(org, torch), to_dev(d, torch)
        _native.call("dm_search_bvh3_first_intersection_ray", torch.cuda.current_stream().cuda_stream, n,
                     o_dev.data_ptr(), d_dev.data_ptr(), hit.data_ptr(), t.data_ptr(), None, T, s_tri.data_ptr(), V,
                     s_vtx.data_ptr(), sbvh.data_ptr(), saabb.data_ptr(), scr.data_ptr(), cs)
        handed = int(scr[4:8].view(torch.int32).item())  # rays handed to the warp tier
        assert handed > 100
        assert np.array_equal(to_np(hit, torch).view(np.uint32), r_hit)
        assert np.array_equal(bits(to_np(t, torch)), bits(r_t))
    finally:
        _native.set_tuning(**before)
    assert _native.device_status(clear=True) == 0
