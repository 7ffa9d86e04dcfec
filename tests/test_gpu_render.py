"""Depth and attribute interpolation from a pix2tri image on the GPU against
the oracle: forward passes bit-exact, backward passes (atomic accumulation,
as the reference's kernels) within float reassociation of the sequential
sums."""
import numpy as np
import pytest

from helpers import bits, to_dev, to_np

from del_msh_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _scene(torch, oracle, ndiv, img_w, img_h, seed):
    from del_msh_gb300.Pix2Tri import torch as Pix2Tri
    from del_msh_gb300.TriMesh3 import torch as TriMesh3
    tri, vtx = W.displaced_torus(ndiv, seed=seed)
    m = W.pinhole_ndc2world(W.random_viewpoint(3.0, seed=seed), aspect=img_w / img_h)
    d_tri, d_vtx = to_dev(tri, torch), to_dev(vtx, torch)
    bvh, aabb = TriMesh3.make_bvhnodes_bvhnode2aabb(d_tri, d_vtx)
    m_row = torch.from_numpy(np.ascontiguousarray(m.reshape(4, 4).T)).to("cuda:0")
    p2t = Pix2Tri.by_raycasting(d_tri, d_vtx, bvh, aabb, m_row, (img_w, img_h))
    return tri, vtx, m, d_tri, d_vtx, m_row, p2t


def _close_sum(got, ref):
    """Sums of the same terms in another order: relative 1e-5 of the largest
    entry (the sums here have at most a few hundred terms)."""
    scale = max(float(np.abs(ref).max()), 1e-30)
    return np.allclose(got, ref, rtol=1e-5, atol=1e-5 * scale)


@pytest.mark.parametrize("ndiv,img", [(64, (96, 72)), (256, (640, 480))])
def test_pix2depth_fwd_bwd(cuda, oracle, ndiv, img):
    torch = cuda
    from del_msh_gb300 import _native
    from del_msh_gb300.Pix2Depth import torch as Pix2Depth
    img_w, img_h = img
    tri, vtx, m, d_tri, d_vtx, m_row, p2t = _scene(torch, oracle, ndiv, img_w, img_h, 7)
    h_p2t = to_np(p2t, torch)
    assert (h_p2t != 0xFFFFFFFF).sum() > img_w * img_h // 10
    depth = torch.zeros((img_h, img_w), dtype=torch.float32, device="cuda:0")
    Pix2Depth.update(depth, p2t, d_tri, d_vtx, m_row)
    ref = oracle.pix2depth(h_p2t, tri, vtx, m, img_w, img_h)
    assert np.array_equal(bits(to_np(depth, torch)), bits(ref))
    g = np.random.default_rng(1).random((img_h, img_w)).astype(np.float32)
    grad = torch.zeros((vtx.shape[0], 3), dtype=torch.float32, device="cuda:0")
    Pix2Depth.bwd_wrt_vtx2xyz(grad, p2t, d_tri, d_vtx, to_dev(g, torch), m_row)
    rgrad = oracle.pix2depth_bwd(h_p2t, tri, vtx, g, m, img_w, img_h)
    assert np.abs(rgrad).max() > 0
    assert _close_sum(to_np(grad, torch), rgrad)
    # autograd front-end: the same gradient
    v = d_vtx.clone().requires_grad_(True)
    (Pix2Depth.AutogradFunction.apply(v, p2t, d_tri, m_row) * to_dev(g, torch)).sum().backward()
    assert _close_sum(to_np(v.grad, torch), rgrad)
    # the interpolation-named helper is the same differentiable function
    v2 = d_vtx.clone().requires_grad_(True)
    d2 = Pix2Depth.pix2depth_using_interpolation(v2, p2t, d_tri, m_row)
    assert np.array_equal(bits(to_np(d2.detach(), torch)), bits(ref))
    (d2 * to_dev(g, torch)).sum().backward()
    assert _close_sum(to_np(v2.grad, torch), rgrad)
    assert _native.device_status(clear=True) == 0


@pytest.mark.parametrize("ndiv,img,nd", [(64, (96, 72), 1), (256, (640, 480), 3)])
def test_interpolate_fwd_bwd(cuda, oracle, ndiv, img, nd):
    torch = cuda
    from del_msh_gb300 import _native
    from del_msh_gb300.Pix2Tri import torch as Pix2Tri
    img_w, img_h = img
    tri, vtx, m, d_tri, d_vtx, m_row, p2t = _scene(torch, oracle, ndiv, img_w, img_h, 8)
    h_p2t = to_np(p2t, torch)
    val = np.random.default_rng(2).random((vtx.shape[0], nd)).astype(np.float32)
    d_val = to_dev(val, torch)
    pv = Pix2Tri.interpolate_fwd(p2t, d_tri, d_vtx, d_val, m_row)
    ref = oracle.interpolate(h_p2t, tri, vtx, val, m, img_w, img_h)
    assert np.array_equal(bits(to_np(pv, torch)), bits(ref))
    G = np.random.default_rng(3).random((img_h, img_w, nd)).astype(np.float32)
    gx = torch.zeros((vtx.shape[0], 3), dtype=torch.float32, device="cuda:0")
    gv = torch.zeros((vtx.shape[0], nd), dtype=torch.float32, device="cuda:0")
    Pix2Tri.interpolate_bwd(p2t, d_tri, d_vtx, d_val, m_row, to_dev(G, torch), gx, gv)
    rx, rv = oracle.interpolate_bwd(h_p2t, tri, vtx, val, m, G, img_w, img_h)
    assert _close_sum(to_np(gx, torch), rx)
    assert _close_sum(to_np(gv, torch), rv)
    v = d_vtx.clone().requires_grad_(True)
    w = d_val.clone().requires_grad_(True)
    (Pix2Tri.interpolate(p2t, d_tri, v, w, m_row) * to_dev(G, torch)).sum().backward()
    assert _close_sum(to_np(v.grad, torch), rx)
    assert _close_sum(to_np(w.grad, torch), rv)
    assert _native.device_status(clear=True) == 0


def test_pix2depth_singular_transform_sets_status(cuda, oracle):
    torch = cuda
    from del_msh_gb300 import _native
    from del_msh_gb300.Pix2Depth import torch as Pix2Depth
    tri, vtx, m, d_tri, d_vtx, m_row, p2t = _scene(torch, oracle, 32, 40, 30, 9)
    depth = torch.zeros((30, 40), dtype=torch.float32, device="cuda:0")
    zero = torch.zeros((4, 4), dtype=torch.float32, device="cuda:0")
    _native.device_status(clear=True)
    Pix2Depth.update(depth, p2t, d_tri, d_vtx, zero)
    assert _native.device_status(clear=True) & 8
