"""GPU parity of BVH ray casting: hit triangle ids and hit t bit-exact to the
oracle (del-msh-cpu's near-first recursive search), plus the reference's own
property tests and the full-size configurations."""
import math

import numpy as np
import pytest

from helpers import bits, lattice_rays, to_dev, to_np, voxel_cubes

from del_msh_gb300 import workloads as W

pytestmark = pytest.mark.gpu
UMAX = 0xFFFFFFFF


def _dev_mesh(torch, tri, vtx):
    from del_msh_gb300.TriMesh3 import torch as TriMesh3
    d_tri, d_vtx = to_dev(tri, torch), to_dev(vtx, torch)
    bvh, aabb = TriMesh3.make_bvhnodes_bvhnode2aabb(d_tri, d_vtx)
    return d_tri, d_vtx, bvh, aabb


def _cast_pixels(torch, mesh, m_colmajor, w, h):
    from del_msh_gb300.Pix2Tri import torch as Pix2Tri
    m_rowmajor = np.ascontiguousarray(np.asarray(m_colmajor, np.float32).reshape(4, 4).T)
    p2t, tt = Pix2Tri.by_raycasting(*mesh, to_dev(m_rowmajor, torch), (w, h), return_depth=True)
    return to_np(p2t, torch), to_np(tt, torch)


def _status():
    from del_msh_gb300 import _native
    return _native.device_status(clear=True)


def test_cast_icosphere1280_matches_golden(cuda, golden_dir):
    torch = cuda
    g = np.load(golden_dir / "oracle_icosphere1280_256.npz")
    mesh = _dev_mesh(torch, g["tri2vtx"], g["vtx2xyz"])
    p2t, tt = _cast_pixels(torch, mesh, g["ndc2world"], 256, 256)
    assert np.array_equal(p2t, g["pix2tri"])
    assert np.array_equal(bits(tt), bits(g["pix2t"]))
    assert _status() == 0


def test_cast_pinhole_torus_matches_oracle(cuda, oracle):
    torch = cuda
    tri, vtx = W.displaced_torus(256, seed=11)
    ref = oracle.build(tri, vtx)
    m = W.pinhole_ndc2world(W.random_viewpoint(3.0, seed=11), aspect=16 / 9)
    mesh = _dev_mesh(torch, tri, vtx)
    p2t, tt = _cast_pixels(torch, mesh, m, 480, 270)
    r_p2t, r_tt = oracle.pix2tri(tri, vtx, ref["bvhnodes"], ref["bvhnode2aabb"], m, 480, 270)
    assert (p2t != UMAX).mean() > 0.05
    assert np.array_equal(p2t, r_p2t)
    assert np.array_equal(bits(tt), bits(r_tt))
    assert _status() == 0


def test_cast_rays_duplicate_soup_deep_tiers(cuda, oracle):
    """Clustered soup: duplicate Morton codes make chains deeper than the
    on-chip stack, so the overflow tiers run; ids and t stay bit-exact."""
    torch = cuda
    from del_msh_gb300.SearchBvh3 import torch as SearchBvh3
    tri, vtx = W.clustered_soup(300_000, num_cluster=8, seed=12)
    ref = oracle.build(tri, vtx)
    assert oracle.tree_height(ref["bvhnodes"], tri.shape[0]) > 70
    org, d = W.cube_boundary_rays(60_000, seed=12)
    # aim a third of the rays at cluster centroids so they go deep
    cen = oracle.tri2cntr(tri, vtx)[np.random.default_rng(0).integers(0, tri.shape[0], 20_000)]
    d[:20_000] = cen - org[:20_000]
    d = d.astype(np.float32)
    mesh = _dev_mesh(torch, tri, vtx)
    hit, t, bc = SearchBvh3.first_intersection_ray(to_dev(org, torch), to_dev(d, torch), *mesh, return_bc=True)
    r_hit, r_t = oracle.cast_rays(org, d, tri, vtx, ref["bvhnodes"], ref["bvhnode2aabb"])
    assert (r_hit != UMAX).sum() > 1000
    assert np.array_equal(to_np(hit, torch), r_hit)
    assert np.array_equal(bits(to_np(t, torch)), bits(r_t))
    bc = to_np(bc, torch)
    ok = r_hit != UMAX
    assert np.allclose(bc[ok].sum(1), 1.0, atol=1e-5)
    assert _status() == 0


def face_tie_cases(num_mesh=40, num_ray=20000):
    """Seeded voxel surfaces with rays aimed at lattice points: hits on
    bounding-box faces and ties in t between triangles.  Where a hit's t
    rounds below its box's entry t, the far-child test must see the near
    child's result alone, as search_bvh3.rs:168-189 does; a test on the
    result folded with the enclosing level's differs on about one ray in
    10^4 of these."""
    for seed in range(num_mesh):
        rng = np.random.default_rng(1000 + seed)
        grid = 3 + seed % 4
        scale = np.float32(0.1 + rng.random())
        tri, vtx = voxel_cubes(rng, grid, int(rng.integers(1, 7)), scale)
        org, d = lattice_rays(rng, grid, scale, num_ray)
        yield tri, vtx, org, d


def test_cast_rays_box_face_ties(cuda, oracle):
    from del_msh_gb300.SearchBvh3 import torch as SearchBvh3
    torch = cuda
    hits = 0
    for tri, vtx, org, d in face_tie_cases():
        ref = oracle.build(tri, vtx)
        mesh = _dev_mesh(torch, tri, vtx)
        assert np.array_equal(to_np(mesh[2], torch), ref["bvhnodes"])
        hit, t = SearchBvh3.first_intersection_ray(to_dev(org, torch), to_dev(d, torch), *mesh)
        r_hit, r_t = oracle.cast_rays(org, d, tri, vtx, ref["bvhnodes"], ref["bvhnode2aabb"])
        hit, t = to_np(hit, torch), to_np(t, torch)
        assert np.array_equal(hit, r_hit)
        assert np.array_equal(bits(t[r_hit != UMAX]), bits(r_t[r_hit != UMAX]))
        hits += int((r_hit != UMAX).sum())
    assert hits > 100000
    assert _status() == 0


def test_sphere_rays_inside_unit_ball(cuda):
    # search_bvh3.rs:247-303
    torch = cuda
    from del_msh_gb300.SearchBvh3 import torch as SearchBvh3
    tri, vtx = W.icosphere(5)
    mesh = _dev_mesh(torch, tri, vtx)
    rng = np.random.default_rng(0)
    n = 1000
    org = np.stack([rng.random(n) * 2 - 1, rng.random(n) * 2 - 1, np.ones(n)], 1).astype(np.float32)
    d = np.tile(np.array([0, 0, -1], np.float32), (n, 1))
    hit, t = SearchBvh3.first_intersection_ray(to_dev(org, torch), to_dev(d, torch), *mesh)
    hit, t = to_np(hit, torch), to_np(t, torch)
    m = hit != UMAX
    p = org[m] + t[m, None] * d[m]
    assert np.all(np.linalg.norm(p, axis=1) < 1.0 + 1e-6)
    assert m.sum() > 600


def test_silhouette_ratio(cuda):
    # del-msh-dlpack/tests/test_trimesh.py:54-99
    torch = cuda
    tri, vtx = W.icosphere(6, radius=0.8)
    mesh = _dev_mesh(torch, tri, vtx)
    p2t, _ = _cast_pixels(torch, mesh, np.eye(4, dtype=np.float32).reshape(-1), 300, 300)
    assert abs(float((p2t != UMAX).mean()) - 0.8 * 0.8 * math.pi * 0.25) < 2e-3


def test_t_error_against_f64(cuda, oracle):
    """FP64 ray/triangle error of the GPU t (which equals the oracle's)."""
    torch = cuda
    g = W.jittered_icosphere(3, seed=0)
    tri, vtx = g
    mesh = _dev_mesh(torch, tri, vtx)
    m = W.ortho_ndc2world()
    p2t, tt = _cast_pixels(torch, mesh, m, 128, 128)
    worst = 0.0
    for i in np.flatnonzero(p2t.reshape(-1) != UMAX)[::7]:
        o, d = oracle.ray_for_pixel(int(i), 128, 128, m)
        it = p2t.reshape(-1)[i]
        t64 = oracle.tri3_ray_f64(vtx[tri[it][0]], vtx[tri[it][1]], vtx[tri[it][2]], o, d)
        worst = max(worst, abs(float(tt.reshape(-1)[i]) - t64) / abs(t64))
    assert worst < 1e-6 * 10  # f32 rounding of the MT formula; reported in the bench


def test_full_torus_2m_1080p(cuda, oracle):
    """2,097,152-triangle displaced torus, 1920x1080 pinhole camera: build
    and cast bit-exact to the oracle at full size."""
    torch = cuda
    tri, vtx = W.displaced_torus(1024, seed=0)
    m = W.pinhole_ndc2world(W.random_viewpoint(3.0, seed=0), aspect=1920 / 1080)
    ref = oracle.build(tri, vtx)
    from del_msh_gb300.TriMesh3 import torch as TriMesh3
    got = TriMesh3.make_bvhnodes_bvhnode2aabb_ex(to_dev(tri, torch), to_dev(vtx, torch))
    assert np.array_equal(to_np(got["bvhnodes"], torch), ref["bvhnodes"])
    assert np.array_equal(bits(to_np(got["bvhnode2aabb"], torch)), bits(ref["bvhnode2aabb"]))
    mesh = (to_dev(tri, torch), to_dev(vtx, torch), got["bvhnodes"], got["bvhnode2aabb"])
    p2t, tt = _cast_pixels(torch, mesh, m, 1920, 1080)
    r_p2t, r_tt = oracle.pix2tri(tri, vtx, ref["bvhnodes"], ref["bvhnode2aabb"], m, 1920, 1080)
    assert np.array_equal(p2t, r_p2t)
    assert np.array_equal(bits(tt), bits(r_tt))
    assert _status() == 0


def test_full_clustered_soup_4m(cuda, oracle):
    """4,194,304-triangle clustered soup with duplicate Morton codes: sort,
    topology and AABBs bit-exact at full size; 1M boundary rays bit-exact."""
    torch = cuda
    from del_msh_gb300.SearchBvh3 import torch as SearchBvh3
    from del_msh_gb300.TriMesh3 import torch as TriMesh3
    tri, vtx = W.clustered_soup(4_194_304, seed=0)
    ref = oracle.build(tri, vtx)
    got = TriMesh3.make_bvhnodes_bvhnode2aabb_ex(to_dev(tri, torch), to_dev(vtx, torch))
    for k in ("idx2tri", "idx2morton", "bvhnodes"):
        assert np.array_equal(to_np(got[k], torch), ref[k]), k
    assert np.array_equal(bits(to_np(got["bvhnode2aabb"], torch)), bits(ref["bvhnode2aabb"]))
    org, d = W.cube_boundary_rays(1_048_576, seed=0)
    mesh = (to_dev(tri, torch), to_dev(vtx, torch), got["bvhnodes"], got["bvhnode2aabb"])
    hit, t = SearchBvh3.first_intersection_ray(to_dev(org, torch), to_dev(d, torch), *mesh)
    r_hit, r_t = oracle.cast_rays(org, d, tri, vtx, ref["bvhnodes"], ref["bvhnode2aabb"])
    assert np.array_equal(to_np(hit, torch), r_hit)
    assert np.array_equal(bits(to_np(t, torch)), bits(r_t))
    assert _status() == 0


def test_cast_equals_rasterisation_reference_pin(cuda, oracle):
    """del-msh-cpu's pixel-level pin (pix2tri.rs:121-173): the GPU's hit
    triangle of every pixel of the 256x256 rotated torus equals the triangle
    rasterised there (pix2tri.rs:50-119, restated in the oracle), and the
    oracle's cast, bit for bit with t."""
    torch = cuda
    from helpers import reference_pin_torus
    tri, vtx, m = reference_pin_torus()
    p2t, tt = _cast_pixels(torch, _dev_mesh(torch, tri, vtx), m, 256, 256)
    ras, _ = oracle.pix2tri_by_rasterization(tri, vtx, m, 256, 256)
    assert (p2t != UMAX).sum() > 10000
    assert np.array_equal(p2t, ras)
    r = oracle.build(tri, vtx)
    r_p2t, r_tt = oracle.pix2tri(tri, vtx, r["bvhnodes"], r["bvhnode2aabb"], m, 256, 256)
    assert np.array_equal(p2t, r_p2t)
    assert np.array_equal(bits(tt), bits(r_tt))
    assert _status() == 0


@pytest.mark.parametrize("name", ["bunny", "spot"])
def test_reference_asset_meshes(cuda, oracle, golden_dir, name):
    """The reference's example meshes (asset/bunny_1k.obj,
    asset/spot/spot_triangulated.obj): build and a 256x256 orthographic cast
    over the mesh's box from +z and a pinhole view, bit-exact to the oracle."""
    torch = cuda
    from del_msh_gb300.TriMesh3 import torch as TriMesh3
    g = np.load(golden_dir / "ref_assets.npz")
    tri, vtx = g[f"{name}__tri2vtx"], g[f"{name}__vtx2xyz"]
    ref = oracle.build(tri, vtx)
    got = TriMesh3.make_bvhnodes_bvhnode2aabb_ex(to_dev(tri, torch), to_dev(vtx, torch))
    assert np.array_equal(to_np(got["bvhnodes"], torch), ref["bvhnodes"])
    assert np.array_equal(bits(to_np(got["bvhnode2aabb"], torch)), bits(ref["bvhnode2aabb"]))
    mesh = (to_dev(tri, torch), to_dev(vtx, torch), got["bvhnodes"], got["bvhnode2aabb"])
    lo, hi = vtx.min(0), vtx.max(0)
    centre = (lo + hi) / 2
    cams = [W.box_ortho_ndc2world(lo, hi),
            W.pinhole_ndc2world(centre + 2.5 * float((hi - lo).max()) * np.array([0.3, 0.4, 0.866]), target=centre,
                                up=(0, 1, 0), aspect=1.0)]
    for m in cams:
        p2t, tt = _cast_pixels(torch, mesh, m, 256, 256)
        r_p2t, r_tt = oracle.pix2tri(tri, vtx, ref["bvhnodes"], ref["bvhnode2aabb"], m, 256, 256)
        assert (p2t != UMAX).sum() > 2000
        assert np.array_equal(p2t, r_p2t)
        assert np.array_equal(bits(tt), bits(r_tt))
    assert _status() == 0
