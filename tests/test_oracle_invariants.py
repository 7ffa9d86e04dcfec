"""Reference test strategy on the oracle: sortedness and topology invariants
(bvhnodes_morton.rs:52-107), the sphere ray test (search_bvh3.rs:247-303),
silhouette area (test_trimesh.py:54-99) and root AABB (test_bvh.py:10-20)."""
import math

import numpy as np
import pytest

from del_msh_gb300 import workloads as W


@pytest.mark.parametrize("seed", [0, 1])
def test_topology_invariants_random_points(oracle, seed):
    rng = np.random.default_rng(seed)
    pts = rng.random((100_000, 3)).astype(np.float32)
    codes = oracle.vtx2morton(pts, np.eye(4, dtype=np.float32).reshape(-1))
    idx, srt = oracle.argsort_stable(codes)
    assert np.all(srt[:-1] <= srt[1:])
    assert oracle.check_morton_code_range_split(srt)
    bvh = oracle.update_bvhnodes(idx, srt)
    assert oracle.check_bvh_topology(bvh, pts.shape[0])


def test_topology_invariants_2d(oracle):
    rng = np.random.default_rng(3)
    pts = rng.random((100_000, 2)).astype(np.float32)
    codes = oracle.vtx2morton(pts, np.eye(3, dtype=np.float32).reshape(-1))
    idx, srt = oracle.argsort_stable(codes)
    bvh = oracle.update_bvhnodes(idx, srt)
    assert oracle.check_bvh_topology(bvh, pts.shape[0])


def test_duplicate_heavy_soup(oracle):
    tri, vtx = W.clustered_soup(60_000, seed=2)
    r = oracle.build(tri, vtx)
    assert oracle.check_bvh_topology(r["bvhnodes"], tri.shape[0])
    assert oracle.check_morton_code_range_split(r["idx2morton"])
    assert oracle.tree_height(r["bvhnodes"], tri.shape[0]) > 50  # duplicate runs make chains


def test_first_intersection_on_sphere(oracle):
    # search_bvh3.rs:247-303: rays along -z at a sphere; the hit lies inside
    # the unit ball and every crossing ray meets exactly two triangles.
    tri, vtx = W.icosphere(5)
    r = oracle.build(tri, vtx)
    rng = np.random.default_rng(0)
    n = 1000
    org = np.stack([rng.random(n) * 2 - 1, rng.random(n) * 2 - 1, np.ones(n)], 1).astype(np.float32)
    d = np.tile(np.array([0, 0, -1], np.float32), (n, 1))
    hit, t = oracle.cast_rays(org, d, tri, vtx, r["bvhnodes"], r["bvhnode2aabb"], threads=4)
    for i in range(n):
        ht, hi, cnt = oracle.intersections_ray(org[i], d[i], tri, vtx, r["bvhnodes"], r["bvhnode2aabb"])
        if hit[i] != 0xFFFFFFFF:
            p = org[i] + t[i] * d[i]
            assert np.linalg.norm(p) < 1.0 + 1e-6
            assert cnt == 2 and (ht[0] == t[i] or ht[1] == t[i])
        else:
            assert cnt == 0


def test_silhouette_ratio(oracle):
    # test_trimesh.py:54-99: sphere of radius 0.8 with the identity ndc2world
    tri, vtx = W.icosphere(6, radius=0.8)
    r = oracle.build(tri, vtx)
    p2t, _ = oracle.pix2tri(tri, vtx, r["bvhnodes"], r["bvhnode2aabb"], np.eye(4, dtype=np.float32).reshape(-1),
                            300, 300, want_t=False)
    ratio = float((p2t != 0xFFFFFFFF).mean())
    assert abs(ratio - 0.8 * 0.8 * math.pi * 0.25) < 2e-3


def test_root_aabb_of_sphere(oracle):
    # del-msh-numpy/tests/test_bvh.py:10-20
    tri, vtx = W.icosphere(3)
    r = oracle.build(tri, vtx)
    assert np.abs(r["bvhnode2aabb"][0] - np.array([-1, -1, -1, 1, 1, 1])).max() < 1e-2
    ref = np.concatenate([vtx.min(0), vtx.max(0)])
    assert np.array_equal(r["bvhnode2aabb"][0], ref)


def test_t_error_against_f64(oracle):
    """Relative error of the f32 hit coefficient against the same formula in
    binary64, on the 1280-triangle icosphere."""
    tri, vtx = W.jittered_icosphere(3, seed=0)
    r = oracle.build(tri, vtx)
    m = W.ortho_ndc2world()
    p2t, tt = oracle.pix2tri(tri, vtx, r["bvhnodes"], r["bvhnode2aabb"], m, 64, 64)
    worst = 0.0
    for i in np.flatnonzero(p2t.reshape(-1) != 0xFFFFFFFF):
        o, d = oracle.ray_for_pixel(int(i), 64, 64, m)
        it = p2t.reshape(-1)[i]
        t64 = oracle.tri3_ray_f64(vtx[tri[it][0]], vtx[tri[it][1]], vtx[tri[it][2]], o, d)
        worst = max(worst, abs(float(tt.reshape(-1)[i]) - t64) / abs(t64))
    assert worst < 1e-5


def test_chain_link_boxes_are_suffix_unions(oracle):
    """On a duplicate-heavy soup, every chain link j (leaf j left, branch j + 1
    right) has the box from_two_aabbs(leaf j, branch j + 1), i.e. the
    first-wins union of its leaf and the rest of the chain: within a run of
    links the boxes are suffix unions of the sorted leaf boxes, the identity a
    run-wise suffix scan of the refit would rest on."""
    tri, vtx = W.clustered_soup(60_000, num_cluster=4, seed=2)
    r = oracle.build(tri, vtx)
    bvh, box = r["bvhnodes"].astype(np.int64), r["bvhnode2aabb"]
    T = tri.shape[0]
    j = np.arange(T - 1)
    link = (bvh[j, 1] == T - 1 + j) & (bvh[j, 2] == j + 1)
    j = j[link]
    assert j.size > T // 4
    a, b = box[T - 1 + j], box[j + 1]  # leaf j, branch j + 1
    lo = np.where(b[:, :3] < a[:, :3], b[:, :3], a[:, :3])  # the first box wins ties (and -0/+0)
    hi = np.where(b[:, 3:] > a[:, 3:], b[:, 3:], a[:, 3:])
    want = np.concatenate([lo, hi], axis=1)
    assert np.array_equal(box[j].view(np.uint32), want.astype(np.float32).view(np.uint32))


def _leftmost_fold(leaves):
    """Fold of boxes [n, 6] with the refit's union (keep the running box's
    component unless the next one is strictly smaller / larger): per
    component, the first leaf that attains the extreme, its bits included."""
    lo, hi = leaves[:, :3], leaves[:, 3:]
    first_lo = np.argmax(lo == lo.min(axis=0), axis=0)
    first_hi = np.argmax(hi == hi.max(axis=0), axis=0)
    return np.concatenate([lo[first_lo, np.arange(3)], hi[first_hi, np.arange(3)]])


def test_run_branches_split_at_a_window_edge(oracle):
    """The identity the refit's run path rests on (1024-leaf windows, as the
    kernels use): where a run of equal codes crosses a window's right edge,
    the window's last branch ends at the run's end b*, and every branch whose
    range [a, b*] starts inside that window has the box union(fold(a ..
    wEnd), fold(wEnd + 1 .. b*)) in leaf order, bit for bit (-0/+0 ties
    included), as the oracle's recursion computes it."""
    tri, vtx = W.clustered_soup(60_000, num_cluster=4, seed=2)
    r = oracle.build(tri, vtx)
    bvh, box = r["bvhnodes"].astype(np.int64), r["bvhnode2aabb"]
    T = tri.shape[0]
    # leaf range of every node, children before parents (explicit post-order)
    lo, hi = np.zeros(2 * T - 1, np.int64), np.zeros(2 * T - 1, np.int64)
    lo[T - 1:] = hi[T - 1:] = np.arange(T)
    stack, order = [0], []
    while stack:
        n = stack.pop()
        order.append(n)
        if n < T - 1:
            stack += [int(bvh[n, 1]), int(bvh[n, 2])]
    for n in reversed(order):
        if n < T - 1:
            c0, c1 = bvh[n, 1], bvh[n, 2]
            lo[n], hi[n] = min(lo[c0], lo[c1]), max(hi[c0], hi[c1])
    leaves = box[T - 1:]
    win, checked, windows_with_runs = 1024, 0, 0
    for w0 in range(0, T - 1, win):
        w_end = w0 + win - 1
        if w_end >= T - 1:
            break
        if not (lo[w_end] >= w0 and hi[w_end] > w_end):
            continue
        bstar = hi[w_end]
        g = np.arange(w0, w_end + 1)
        run = g[(lo[g] >= w0) & (hi[g] == bstar)]
        if run.size < 64:
            continue
        windows_with_runs += 1
        right = _leftmost_fold(leaves[w_end + 1:bstar + 1])
        for n in run:
            left = _leftmost_fold(leaves[lo[n]:w_end + 1])
            both = _leftmost_fold(np.stack([left, right]))
            assert np.array_equal(box[n].view(np.uint32), both.astype(np.float32).view(np.uint32)), (w0, n)
            checked += 1
    assert windows_with_runs >= 8 and checked >= 512
