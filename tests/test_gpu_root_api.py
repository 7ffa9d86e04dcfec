"""The package-root entry points (del_msh_dlpack's DLPack-level functions:
TriMesh3.make_bvhnode2aabb_from_bvhnodes, Pix2Tri.update_pix2tri /
interpolate / interpolate_bwd) give the torch front-ends' results, on the
default stream (stream_ptr=0) and on a side stream, with DLPack inputs."""
import numpy as np
import pytest

from helpers import bits, to_dev, to_np

from del_msh_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("side_stream", [False, True])
def test_root_functions_match_torch_front_end(cuda, side_stream):
    torch = cuda
    import del_msh_gb300.Pix2Tri as RootPix2Tri
    import del_msh_gb300.TriMesh3 as RootTriMesh3
    from del_msh_gb300 import _native
    from del_msh_gb300.Pix2Tri import torch as Pix2Tri
    from del_msh_gb300.TriMesh3 import torch as TriMesh3
    tri, vtx = W.jittered_icosphere(4, seed=9)
    d_tri, d_vtx = to_dev(tri, torch), to_dev(vtx, torch)
    bvh, aabb = TriMesh3.make_bvhnodes_bvhnode2aabb(d_tri, d_vtx)
    m_row = torch.from_numpy(W.ortho_ndc2world().reshape(4, 4).T.copy()).to("cuda:0")
    want_p2t = Pix2Tri.by_raycasting(d_tri, d_vtx, bvh, aabb, m_row, (96, 80))
    val = to_dev(np.random.default_rng(3).random((vtx.shape[0], 2)).astype(np.float32), torch)
    want_val = Pix2Tri.interpolate_fwd(want_p2t, d_tri, d_vtx, val, m_row)
    torch.cuda.synchronize()
    s = torch.cuda.Stream() if side_stream else None
    sp = s.cuda_stream if s is not None else 0
    aabb2 = torch.empty_like(aabb)
    RootTriMesh3.make_bvhnode2aabb_from_bvhnodes(d_tri, d_vtx.__dlpack__(), None, bvh, aabb2, stream_ptr=sp)
    p2t = torch.empty((80, 96), dtype=torch.uint32, device="cuda:0")
    colmajor = m_row.T.contiguous()
    RootPix2Tri.update_pix2tri(d_tri, d_vtx, bvh, aabb2, colmajor, p2t, stream_ptr=sp)
    pv = torch.zeros((80, 96, 2), dtype=torch.float32, device="cuda:0")
    RootPix2Tri.interpolate(p2t, d_tri, d_vtx, val, colmajor, pv, stream_ptr=sp)
    g = torch.ones_like(pv)
    gx, gv = torch.zeros_like(d_vtx), torch.zeros_like(val)
    RootPix2Tri.interpolate_bwd(p2t, d_tri, d_vtx, val, colmajor, g, gx, gv, stream_ptr=sp)
    torch.cuda.synchronize()
    assert np.array_equal(bits(to_np(aabb2, torch)), bits(to_np(aabb, torch)))
    assert np.array_equal(to_np(p2t, torch), to_np(want_p2t, torch))
    assert np.array_equal(bits(to_np(pv, torch)), bits(to_np(want_val, torch)))
    assert float(gv.abs().sum()) > 0
    assert _native.device_status(clear=True) == 0
