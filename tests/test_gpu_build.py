"""GPU parity of the LBVH build stages against the oracle and the reference's
own golden vectors.  Integer results and f32 AABBs are compared bit for bit."""
import numpy as np
import pytest

from helpers import bits, to_dev, to_np

from del_msh_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _status_clear():
    from del_msh_gb300 import _native
    return _native.device_status(clear=True)


def test_morton_points_match_reference_code(cuda, oracle, golden_dir):
    """Finite points through the identity transform give the reference's own
    morton_code3 values; every point (NaN / inf included, where 0*inf makes
    the homogeneous w NaN) gives the oracle's value."""
    torch = cuda
    from del_msh_gb300.Mortons import torch as Mortons
    g = np.load(golden_dir / "ref_morton.npz")
    got = to_np(Mortons.make_vtx2morton_from_vtx2co(to_dev(g["pts"], torch), torch.eye(4, device="cuda:0")), torch)
    finite = np.isfinite(g["pts"]).all(1)
    assert np.array_equal(got[finite], g["codes"][finite])
    assert np.array_equal(got, oracle.vtx2morton(g["pts"], np.eye(4, dtype=np.float32).reshape(-1)))


@pytest.mark.parametrize("dim", [2, 3])
def test_morton_points_with_transform(cuda, oracle, dim):
    # del-msh-dlpack/tests/test_mortons.py:64-98 (a transform vs pre-transformed points)
    torch = cuda
    from del_msh_gb300.Mortons import torch as Mortons
    rng = np.random.default_rng(dim)
    pts = (rng.random((20_000, dim)) * 3.0 - 1.0).astype(np.float32)
    m = np.eye(dim + 1, dtype=np.float32)
    m[:dim, :dim] /= 3.0
    m[:dim, dim] = 1.0 / 3.0
    got = to_np(Mortons.make_vtx2morton_from_vtx2co(to_dev(pts, torch), to_dev(m, torch)), torch)
    ref = oracle.vtx2morton(pts, np.ascontiguousarray(m.T).reshape(-1))
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("n", [1, 2, 3, 100, 3839, 3840, 3841, 65_537, 1_000_003])
def test_argsort_stable(cuda, n):
    torch = cuda
    from del_msh_gb300.Array1D import torch as Array1D
    rng = np.random.default_rng(n)
    vals = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    if n > 10:
        vals[rng.random(n) < 0.3] = 0xFFFFFFFF
        vals[rng.random(n) < 0.2] = 7
    idx, srt = Array1D.argsort(to_dev(vals, torch))
    ref = np.argsort(vals, kind="stable").astype(np.uint32)
    assert np.array_equal(to_np(idx, torch), ref)
    assert np.array_equal(to_np(srt, torch), vals[ref])


def test_argsort_all_equal(cuda):
    torch = cuda
    from del_msh_gb300.Array1D import torch as Array1D
    vals = np.full(200_000, 42, np.uint32)
    idx, srt = Array1D.argsort(to_dev(vals, torch))
    assert np.array_equal(to_np(idx, torch), np.arange(200_000, dtype=np.uint32))


def test_topology_matches_reference_code(cuda, golden_dir):
    torch = cuda
    from del_msh_gb300.Mortons import torch as Mortons
    g = np.load(golden_dir / "ref_topology.npz")
    for name in sorted({k.split("__")[0] for k in g.files}):
        got = Mortons.make_bvhnodes_from_sorted_mortons(to_dev(g[f"{name}__idx2obj"], torch),
                                                        to_dev(g[f"{name}__idx2morton"], torch))
        assert np.array_equal(to_np(got, torch), g[f"{name}__bvhnodes"]), name


def test_topology_single_object(cuda):
    torch = cuda
    from del_msh_gb300.Mortons import torch as Mortons
    got = Mortons.make_bvhnodes_from_sorted_mortons(to_dev(np.array([5], np.uint32), torch),
                                                    to_dev(np.array([77], np.uint32), torch))
    assert to_np(got, torch).tolist() == [[0xFFFFFFFF, 5, 0xFFFFFFFF]]


def _build_ex(torch, tri, vtx, want_height=True):
    from del_msh_gb300.TriMesh3 import torch as TriMesh3
    r = TriMesh3.make_bvhnodes_bvhnode2aabb_ex(to_dev(tri, torch), to_dev(vtx, torch), want_height=want_height)
    out = {k: (to_np(v, torch) if hasattr(v, "device") else v) for k, v in r.items()}
    out["transform"] = np.ascontiguousarray(out["transform"].T).reshape(-1)  # back to column-major
    return out


def _compare_build(got, ref, T):
    for k in ("transform", "tri2morton", "idx2tri", "idx2morton", "bvhnodes", "bvhnode2aabb"):
        assert np.array_equal(bits(got[k]), bits(ref[k])), k


def test_build_icosphere1280_matches_golden(cuda, golden_dir):
    torch = cuda
    g = np.load(golden_dir / "oracle_icosphere1280_256.npz")
    got = _build_ex(torch, g["tri2vtx"], g["vtx2xyz"])
    _compare_build(got, {k: g[k] for k in g.files}, g["tri2vtx"].shape[0])
    assert _status_clear() == 0


def signed_zero_mesh(runs: bool):
    """Boxes whose extremes tie between -0.0 and +0.0: a box keeps the
    leftmost extreme (the first vertex of a triangle, the leftmost leaf of a
    branch), so the bits of every refit path must follow that order.
    Grid: 262k triangles on the plane z = ±0 with a column at x = ±0 (window
    heaps, superblocks, 8-lane crossing queries).  Runs: 64 clusters of 10k
    triangles on the plane x = ±0 whose centroids share Morton codes, so the
    runs cross many windows (more crossing branches than 8-lane groups: the
    one-thread crossing kernel)."""
    if not runs:
        rng = np.random.default_rng(9)
        nx, ny = 513, 257
        gx, gy = np.meshgrid(np.linspace(-1, 1, nx), np.linspace(0, 1, ny), indexing="ij")
        vtx = np.stack([gx, gy, np.zeros_like(gx)], -1).reshape(-1, 3).astype(np.float32)
        zero = np.where(rng.random(vtx.shape) < 0.5, np.float32(-0.0), np.float32(0.0)).astype(np.float32)
        vtx = np.where(vtx == 0, zero, vtx).astype(np.float32)
        i, j = np.meshgrid(np.arange(nx - 1), np.arange(ny - 1), indexing="ij")
        v00 = (i * ny + j).ravel()
        v10, v01, v11 = v00 + ny, v00 + 1, v00 + ny + 1
        tri = np.stack([np.stack([v00, v10, v11], 1), np.stack([v00, v11, v01], 1)], 1).reshape(-1, 3)
        return tri.astype(np.uint32), vtx
    rng = np.random.default_rng(10)
    k, m = 64, 10_000
    c = rng.random((k, 1, 2)).astype(np.float32)
    e = (rng.random((k, m, 1)) * 1e-3).astype(np.float32)
    y, z = c[..., 0:1], c[..., 1:2]
    p0 = np.concatenate([np.zeros_like(e), y + e, z + 0 * e], -1)
    p1 = np.concatenate([np.zeros_like(e), y - e, z + 0 * e], -1)
    p2 = np.concatenate([np.zeros_like(e), y + 0 * e, z + e], -1)
    vtx = np.stack([p0, p1, p2], 2).reshape(-1, 3).astype(np.float32)
    vtx[:, 0] = np.where(rng.random(vtx.shape[0]) < 0.5, np.float32(-0.0), np.float32(0.0))
    tri = np.arange(vtx.shape[0], dtype=np.uint32).reshape(-1, 3)
    return tri, vtx


@pytest.mark.parametrize("want_height", [True, False])
@pytest.mark.parametrize("case", ["torus", "soup", "ico", "tiny2", "tiny3", "same_tris", "flat", "nan_vertex",
                                  "big_window_span", "signed_zero_grid", "signed_zero_runs"])
def test_build_matches_oracle(cuda, oracle, case, want_height):
    """Both refits: the tree-order climb (asked for the height) and the range
    queries (no height; NaN in a leaf box hands the call to the climb)."""
    torch = cuda
    if case == "torus":
        tri, vtx = W.displaced_torus(256, seed=3)
    elif case == "soup":
        tri, vtx = W.clustered_soup(200_000, seed=4)
    elif case == "ico":
        tri, vtx = W.jittered_icosphere(5, seed=5)
    elif case == "tiny2":
        tri, vtx = W.icosphere(0)
        tri = tri[:2]
    elif case == "tiny3":
        tri, vtx = W.icosphere(0)
        tri = tri[:3]
    elif case == "same_tris":
        tri = np.tile(np.array([[0, 1, 2]], np.uint32), (5000, 1))
        vtx = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    elif case == "nan_vertex":
        tri, vtx = W.displaced_torus(64, seed=6)
        vtx = vtx.copy()
        vtx[[5, 700, 2047]] = np.nan
    elif case == "big_window_span":  # > 2^15 leaves: superblock and top heaps, ragged last window
        tri, vtx = W.displaced_torus(190, seed=7)
        tri = tri[:-37]
    elif case.startswith("signed_zero"):
        tri, vtx = signed_zero_mesh(case == "signed_zero_runs")
    else:  # all vertices on the plane z = 0
        rng = np.random.default_rng(8)
        vtx = np.concatenate([rng.random((3000, 2)), np.zeros((3000, 1))], 1).astype(np.float32)
        tri = rng.integers(0, 3000, (4000, 3)).astype(np.uint32)
    ref = oracle.build(tri, vtx)
    got = _build_ex(torch, tri, vtx, want_height)
    _compare_build(got, ref, tri.shape[0])
    if want_height:
        assert got["height"] == oracle.tree_height(ref["bvhnodes"], tri.shape[0])
    assert _status_clear() == 0


@pytest.mark.parametrize("want_height", [False, True])
def test_full_torus_8m_build(cuda, oracle, want_height):
    """8,388,608-triangle displaced torus: above the cooperative front's
    capacity, so the separate kernels build it (centroid pass with the fit
    transform, Morton codes with the digit histograms, the onesweep passes,
    topology, the refit windows and their crossing branches, or the
    tree-order climb when the height is asked for); every intermediate and
    the tree and boxes bit-exact to the oracle, and a deformed frame through
    the drop-in refit too."""
    torch = cuda
    tri, vtx = W.displaced_torus(2048, seed=1)
    ref = oracle.build(tri, vtx)
    got = _build_ex(torch, tri, vtx, want_height)
    _compare_build(got, ref, tri.shape[0])
    if want_height:
        assert got["height"] == oracle.tree_height(ref["bvhnodes"], tri.shape[0])
    else:
        # a deformed frame through the drop-in refit (leaf ranges derived on
        # the device from bvhnodes alone, then the range queries)
        from del_msh_gb300.TriMesh3 import torch as TriMesh3
        v = (vtx + 0.01 * np.sin(np.random.default_rng(2).uniform(0, 6.28, vtx.shape[0]) + 1.0)[:, None])
        v = v.astype(np.float32)
        bvh = to_dev(got["bvhnodes"], torch)
        aabb = torch.empty((2 * tri.shape[0] - 1, 6), dtype=torch.float32, device="cuda:0")
        TriMesh3.update_bvhnode2aabb(to_dev(tri, torch), to_dev(v, torch), bvh, aabb)
        want = oracle.bvhnode2aabb(ref["bvhnodes"], tri, v)
        assert np.array_equal(bits(to_np(aabb, torch)), bits(want))
    assert _status_clear() == 0


def test_build_single_triangle(cuda):
    torch = cuda
    tri = np.array([[0, 1, 2]], np.uint32)
    vtx = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 2]], np.float32)
    got = _build_ex(torch, tri, vtx)
    assert got["bvhnodes"].tolist() == [[0xFFFFFFFF, 0, 0xFFFFFFFF]]
    assert got["bvhnode2aabb"].tolist() == [[0, 0, 0, 1, 1, 2]]


def test_refit_deformed_and_ccd(cuda, oracle):
    torch = cuda
    from del_msh_gb300.TriMesh3 import torch as TriMesh3
    tri, vtx = W.displaced_torus(128, seed=1)
    ref = oracle.build(tri, vtx)
    d_tri, d_vtx = to_dev(tri, torch), to_dev(vtx, torch)
    bvh, aabb = TriMesh3.make_bvhnodes_bvhnode2aabb(d_tri, d_vtx)
    flags = torch.zeros((tri.shape[0],), dtype=torch.int32, device="cuda:0").view(torch.uint32)
    rng = np.random.default_rng(2)
    phase = rng.uniform(0, 6.28, vtx.shape[0])
    for frame in range(3):
        v1 = (vtx + 0.01 * np.sin(phase + frame)[:, None]).astype(np.float32)
        TriMesh3.update_bvhnode2aabb(d_tri, to_dev(v1, torch), bvh, aabb, flags=flags)
        assert np.array_equal(bits(to_np(aabb, torch)), bits(oracle.bvhnode2aabb(ref["bvhnodes"], tri, v1)))
        assert not to_np(flags, torch).any()  # the refit leaves its arrival flags zero
    v2 = (vtx * 1.01).astype(np.float32)
    TriMesh3.update_bvhnode2aabb(d_tri, d_vtx, bvh, aabb, vtx2xyz1=to_dev(v2, torch))
    assert np.array_equal(bits(to_np(aabb, torch)), bits(oracle.bvhnode2aabb(ref["bvhnodes"], tri, vtx, v2)))
    assert _status_clear() == 0


def _relabel_branches(bvh, seed):
    """The same tree with its branches renumbered at random (root kept at 0):
    still a valid tree, no longer in Karras leaf order."""
    bvh = np.asarray(bvh, np.uint32).reshape(-1, 3)
    nb = (bvh.shape[0] + 1) // 2 - 1
    perm = np.arange(bvh.shape[0], dtype=np.int64)
    perm[1:nb] = 1 + np.random.default_rng(seed).permutation(nb - 1)
    umax = np.uint32(0xFFFFFFFF)
    mapped = np.where(bvh == umax, umax, perm[np.minimum(bvh, bvh.shape[0] - 1)].astype(np.uint32))
    mapped[nb:, 1] = bvh[nb:, 1]  # a leaf's second word is its triangle
    mapped[nb:, 2] = bvh[nb:, 2]
    out = np.empty_like(bvh)
    out[perm] = mapped
    return out


@pytest.mark.parametrize("case", ["torus", "torus_ccd", "soup", "relabelled", "nan", "ex_frames", "ex_soup"])
def test_dropin_refit_paths(cuda, oracle, case):
    """dm_bvhnode2aabb_update_aabb in the reference binding's form (no flag
    scratch): range queries for trees in Karras leaf order (the torus), the
    parent-pointer climb for trees the device cannot show to be (the soup's
    long chains, a tree with its branches renumbered), the tree-order climb
    for NaN leaf boxes; and the _ex form with persistent scratch, frame after
    frame.  Every box equals the oracle's bit for bit."""
    torch = cuda
    from del_msh_gb300 import _native
    from del_msh_gb300.TriMesh3 import torch as TriMesh3
    if case in ("soup", "ex_soup"):
        tri, vtx = W.clustered_soup(150_000, num_cluster=4, seed=3)
    else:
        tri, vtx = W.displaced_torus(96, seed=4)
    ref = oracle.build(tri, vtx)
    bvh_np = _relabel_branches(ref["bvhnodes"], 5) if case == "relabelled" else ref["bvhnodes"]
    d_tri, bvh = to_dev(tri, torch), to_dev(bvh_np, torch)
    T = tri.shape[0]
    aabb = torch.full((2 * T - 1, 6), 7.0, dtype=torch.float32, device="cuda:0")
    phase = np.random.default_rng(6).uniform(0, 6.28, vtx.shape[0])
    L = _native.load()
    ex_scratch = torch.zeros((L.dm_bvhnode2aabb_update_aabb_scratch_bytes(T),), dtype=torch.uint8,
                             device="cuda:0")
    sp = torch.cuda.current_stream().cuda_stream
    for frame in range(3):
        v = (vtx + 0.01 * np.sin(phase + frame)[:, None]).astype(np.float32)
        if case == "nan":
            v[frame * 7 + 1, 1] = np.nan
        v1 = (v * 1.01).astype(np.float32) if case == "torus_ccd" else None
        d_v, d_v1 = to_dev(v, torch), (None if v1 is None else to_dev(v1, torch))
        if case.startswith("ex_"):
            _native.call("dm_bvhnode2aabb_update_aabb_ex", sp, 2 * T - 1, aabb.data_ptr(), bvh.data_ptr(), T,
                         d_tri.data_ptr(), v.shape[0], d_v.data_ptr(), None, ex_scratch.data_ptr(),
                         ex_scratch.numel())
            # the refit header's climb flag (after the derived ends and the
            # arrival words): 0 = range queries, bit 2 = parent-pointer climb
            hdr1 = ((4 * T + 255) // 256 * 256) + 4 * (((T + 3) & ~3) + 1)
            flag = int(ex_scratch[hdr1:hdr1 + 4].cpu().numpy().view(np.uint32)[0])
            assert flag == (0 if case == "ex_frames" else 2), (case, flag)
        else:
            TriMesh3.update_bvhnode2aabb(d_tri, d_v, bvh, aabb, vtx2xyz1=d_v1)
        want = oracle.bvhnode2aabb(bvh_np, tri, v, v1)
        assert np.array_equal(bits(to_np(aabb, torch)), bits(want)), (case, frame)
    assert _status_clear() == 0


def test_cpu_tensors_are_rejected():
    import torch
    from del_msh_gb300.TriMesh3 import torch as TriMesh3
    tri = torch.zeros((1, 3), dtype=torch.uint32)
    vtx = torch.zeros((3, 3), dtype=torch.float32)
    with pytest.raises(NotImplementedError):
        TriMesh3.make_bvhnodes_bvhnode2aabb(tri, vtx)
