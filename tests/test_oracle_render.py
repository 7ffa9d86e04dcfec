"""The oracle's depth / interpolation restatements against an independent
float64 torch computation of the same formulas, differentiated by autograd:
pins the backward derivations (implicit differentiation of the ray-triangle
intersection, the homogeneous-transform Jacobian) without a GPU."""
import numpy as np
import pytest

from del_msh_gb300 import workloads as W

IMG_W, IMG_H = 48, 36


def _scene(oracle):
    tri, vtx = W.displaced_torus(24, seed=5)
    m = W.pinhole_ndc2world(W.random_viewpoint(3.0, seed=4), aspect=IMG_W / IMG_H)
    ref = oracle.build(tri, vtx)
    p2t, _ = oracle.pix2tri(tri, vtx, ref["bvhnodes"], ref["bvhnode2aabb"], m, IMG_W, IMG_H)
    return tri, vtx, m, p2t


def _torch_hits(torch, oracle, tri, vtx_t, m, p2t):
    hit = np.nonzero(p2t.reshape(-1) != 0xFFFFFFFF)[0]
    o = np.empty((hit.size, 3)), np.empty((hit.size, 3))
    for k, i in enumerate(hit):
        org, d = oracle.ray_for_pixel(int(i), IMG_W, IMG_H, m)
        o[0][k], o[1][k] = org, d
    org, d = torch.from_numpy(o[0]), torch.from_numpy(o[1])
    tv_idx = torch.from_numpy(tri[p2t.reshape(-1)[hit]].astype(np.int64))
    p0, p1, p2 = vtx_t[tv_idx[:, 0]], vtx_t[tv_idx[:, 1]], vtx_t[tv_idx[:, 2]]
    e1, e2, tv = p1 - p0, p2 - p0, org - p0
    pv = torch.cross(d, e2, dim=1)
    det = (e1 * pv).sum(1)
    u = (tv * pv).sum(1) / det
    qv = torch.cross(tv, e1, dim=1)
    v = (d * qv).sum(1) / det
    t = (e2 * qv).sum(1) / det
    return hit, tv_idx, org, d, u, v, t


def test_oracle_inverse(oracle):
    rng = np.random.default_rng(0)
    for _ in range(20):
        a = (rng.normal(size=(4, 4)) + 4 * np.eye(4)).astype(np.float32)
        inv, ok = oracle.mat4_inverse_pivot(np.ascontiguousarray(a.T).reshape(-1))
        assert ok
        assert np.allclose(a @ inv.reshape(4, 4).T, np.eye(4), atol=1e-5)
    _, ok = oracle.mat4_inverse_pivot(np.zeros(16, np.float32))
    assert not ok


def test_oracle_depth_and_grad_match_float64_autograd(oracle):
    torch = pytest.importorskip("torch")
    tri, vtx, m, p2t = _scene(oracle)
    w2n, ok = oracle.mat4_inverse_pivot(m)
    assert ok
    depth = oracle.pix2depth(p2t, tri, vtx, m, IMG_W, IMG_H)
    g = np.random.default_rng(1).random((IMG_H, IMG_W)).astype(np.float32)
    grad = oracle.pix2depth_bwd(p2t, tri, vtx, g, m, IMG_W, IMG_H)

    vt = torch.from_numpy(vtx.astype(np.float64)).requires_grad_(True)
    hit, _, org, d, u, v, t = _torch_hits(torch, oracle, tri, vt, m, p2t)
    q = org + t[:, None] * d
    M = torch.from_numpy(w2n.reshape(4, 4).T.astype(np.float64))
    qh = torch.cat([q, torch.ones_like(q[:, :1])], 1) @ M.T
    dep = (qh[:, 2] / qh[:, 3] + 1) * 0.5
    assert np.allclose(depth.reshape(-1)[hit], dep.detach().numpy(), rtol=1e-5, atol=1e-6)
    assert (depth.reshape(-1)[p2t.reshape(-1) == 0xFFFFFFFF] == 0).all()
    (torch.from_numpy(g.reshape(-1)[hit].astype(np.float64)) * dep).sum().backward()
    ref = vt.grad.numpy()
    assert np.abs(ref).max() > 0
    # f32 restatement against float64 autograd: tolerance of the f32 arithmetic
    assert np.allclose(grad, ref, rtol=1e-3, atol=1e-4 * np.abs(ref).max())


def test_oracle_interpolation_and_grad_match_float64_autograd(oracle):
    torch = pytest.importorskip("torch")
    tri, vtx, m, p2t = _scene(oracle)
    val = np.random.default_rng(2).random((vtx.shape[0], 2)).astype(np.float32)
    pv = oracle.interpolate(p2t, tri, vtx, val, m, IMG_W, IMG_H)
    G = np.random.default_rng(3).random((IMG_H, IMG_W, 2)).astype(np.float32)
    gx, gv = oracle.interpolate_bwd(p2t, tri, vtx, val, m, G, IMG_W, IMG_H)

    vt = torch.from_numpy(vtx.astype(np.float64)).requires_grad_(True)
    valt = torch.from_numpy(val.astype(np.float64)).requires_grad_(True)
    hit, tv_idx, _, _, u, v, _ = _torch_hits(torch, oracle, tri, vt, m, p2t)
    out = (1 - u - v)[:, None] * valt[tv_idx[:, 0]] + u[:, None] * valt[tv_idx[:, 1]] + v[:, None] * valt[tv_idx[:, 2]]
    # f32 barycentrics against float64: grazing rays lose a few ulps of u, v
    assert np.allclose(pv.reshape(-1, 2)[hit], out.detach().numpy(), rtol=1e-4, atol=2e-5)
    assert (pv.reshape(-1, 2)[p2t.reshape(-1) == 0xFFFFFFFF] == 0).all()
    (torch.from_numpy(G.reshape(-1, 2)[hit].astype(np.float64)) * out).sum().backward()
    rx, rv = vt.grad.numpy(), valt.grad.numpy()
    assert np.allclose(gx, rx, rtol=1e-3, atol=1e-4 * np.abs(rx).max())
    assert np.allclose(gv, rv, rtol=1e-4, atol=1e-5 * np.abs(rv).max())
