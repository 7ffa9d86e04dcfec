"""Quad/oct-trees from sorted unique Morton codes: the oracle against the
reference's own invariant checker (restated), and the GPU bit for bit
against the oracle (the aggregation, added with atomics, within float
reassociation)."""
import numpy as np
import pytest

from helpers import bits, to_dev, to_np


def _codes(oracle, n, nd, seed, clustered=False):
    rng = np.random.default_rng(seed)
    pts = rng.random((n, nd)).astype(np.float32)
    if clustered:
        pts = (0.5 + 0.01 * rng.standard_normal((n, nd))).clip(0, 1).astype(np.float32)
    codes = oracle.vtx2morton(pts, np.eye(nd + 1, dtype=np.float32).reshape(-1))
    return np.unique(codes)


@pytest.mark.parametrize("nd", [2, 3])
@pytest.mark.parametrize("n,clustered", [(10, False), (3000, False), (20000, True)])
def test_oracle_octree_invariants(oracle, nd, n, clustered):
    u = _codes(oracle, n, nd, 5, clustered)
    t = oracle.quad_oct_tree(u, nd)
    assert oracle.quad_oct_tree_check(t, nd)
    agg = oracle.quad_oct_tree_aggregate(np.ones((u.size, 1), np.float32), t["idx2onode"], t["onodes"])
    assert agg[0, 0] == u.size  # the root holds every leaf


@pytest.mark.gpu
@pytest.mark.parametrize("nd", [2, 3])
@pytest.mark.parametrize("n,clustered", [(10, False), (5000, False), (200_000, True), (1_000_000, False)])
def test_gpu_octree_matches_oracle(cuda, oracle, nd, n, clustered):
    torch = cuda
    from del_msh_gb300 import _native
    from del_msh_gb300.QuadOctTree import torch as QOT
    u = _codes(oracle, n, nd, 7, clustered)
    ref = oracle.quad_oct_tree(u, nd)
    d = to_dev(u, torch)
    bn, b2d, b2o, i2b = QOT.bnodes_and_bnode2depth_and_bnode2onode_and_idx2bnode(d, nd)
    assert np.array_equal(to_np(bn, torch), ref["bnodes"])
    assert np.array_equal(to_np(b2d, torch), ref["bnode2depth"])
    assert np.array_equal(to_np(b2o, torch), ref["bnode2onode"])
    assert np.array_equal(to_np(i2b, torch), ref["idx2bnode"])
    on, o2d, o2c, i2o, i2c = QOT.make_tree_from_binary_radix_tree(bn, b2o, b2d, i2b, d, nd)
    assert np.array_equal(to_np(on, torch), ref["onodes"])
    assert np.array_equal(to_np(o2d, torch), ref["onode2depth"])
    assert np.array_equal(bits(to_np(o2c, torch)), bits(ref["onode2center"]))
    assert np.array_equal(to_np(i2o, torch), ref["idx2onode"])
    assert np.array_equal(bits(to_np(i2c, torch)), bits(ref["idx2center"]))
    val = np.random.default_rng(1).random((u.size, 2)).astype(np.float32)
    agg = to_np(QOT.aggregate(to_dev(val, torch), i2o, on), torch)
    ragg = oracle.quad_oct_tree_aggregate(val, ref["idx2onode"], ref["onodes"])
    # positive sums of up to 1M terms added in another order: a few 1e-5 relative
    assert np.allclose(agg, ragg, rtol=2e-4, atol=1e-6 * np.abs(ragg).max())
    assert _native.device_status(clear=True) == 0
