"""Self-intersection through the BVH (trimesh3_intersection.rs): the oracle's
BVH search equals its brute force and finds nothing on a sphere (the
reference's own test), and the GPU finds the oracle's pairs and segments bit
for bit (as a set: the GPU list is unordered)."""
import numpy as np
import pytest

from helpers import bits, to_dev, to_np

from del_msh_gb300 import workloads as W


def _two_spheres(level, shift):
    t, v = W.icosphere(level)
    t2 = np.concatenate([t, t + v.shape[0]]).astype(np.uint32)
    v2 = np.concatenate([v, v + np.asarray(shift, np.float32)]).astype(np.float32)
    return t2, v2


def _crumpled(level, jitter, seed):
    return W.jittered_icosphere(level, jitter=jitter, seed=seed)


def _sorted(pairs, segs):
    order = np.lexsort((pairs[:, 1], pairs[:, 0]))
    return pairs[order], segs.reshape(-1, 6)[order]


@pytest.mark.parametrize("case", ["two_spheres", "crumpled"])
def test_oracle_bvh_search_equals_brute_force(oracle, case):
    tri, vtx = _two_spheres(2, (0.6, 0.2, 0.1)) if case == "two_spheres" else _crumpled(2, 0.15, 3)
    r = oracle.build(tri, vtx)
    p, s = oracle.self_intersection(tri, vtx, r["bvhnodes"], r["bvhnode2aabb"])
    pb, sb = oracle.self_intersection(tri, vtx, None, None, brute=True)
    assert len(p) > 0
    key = lambda P: sorted(map(tuple, np.sort(P, axis=1)))
    assert key(p) == key(pb)


def test_oracle_sphere_has_no_self_intersection(oracle):
    # trimesh3_intersection.rs:194-233 (test0)
    tri, vtx = W.icosphere(4)
    r = oracle.build(tri, vtx)
    p, _ = oracle.self_intersection(tri, vtx, r["bvhnodes"], r["bvhnode2aabb"])
    assert len(p) == 0


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["sphere", "two_spheres", "crumpled", "crumpled_big"])
def test_gpu_self_intersection_matches_oracle(cuda, oracle, case):
    torch = cuda
    from del_msh_gb300 import _native
    from del_msh_gb300.TriMesh3 import torch as TriMesh3
    if case == "sphere":
        tri, vtx = W.icosphere(5)
    elif case == "two_spheres":
        tri, vtx = _two_spheres(4, (0.7, 0.1, 0.05))
    elif case == "crumpled":
        tri, vtx = _crumpled(3, 0.2, 5)
    else:
        tri, vtx = _crumpled(5, 0.05, 6)
    d_tri, d_vtx = to_dev(tri, torch), to_dev(vtx, torch)
    bvh, aabb = TriMesh3.make_bvhnodes_bvhnode2aabb(d_tri, d_vtx)
    segs, pairs = TriMesh3.self_intersection(d_tri, d_vtx, bvh, aabb, capacity=16)  # grows as needed
    rp, rs = oracle.self_intersection(tri, vtx, to_np(bvh, torch), to_np(aabb, torch))
    gp, gs = _sorted(to_np(pairs, torch), to_np(segs, torch))
    rp, rs = _sorted(rp, rs)
    assert np.array_equal(gp, rp)
    assert np.array_equal(bits(gs), bits(rs))
    if case != "sphere":
        assert len(gp) > 0
    assert _native.device_status(clear=True) == 0
