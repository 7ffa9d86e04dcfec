"""Package-root form of the pix2tri entry points (the functions of
del_msh_dlpack/Pix2Tri/__init__.py): caller-allocated arrays in, results
written in place, launched on ``stream_ptr`` (0 = the default stream).

Arrays are torch CUDA tensors or objects torch.from_dlpack accepts.  As at
the reference's package root, ``transform_ndc2world`` is already in the
kernels' column-major order (the torch front-end in ``.torch`` transposes a
row-major matrix before calling these) and the image size is pix2tri's
(img_h, img_w) shape."""
from __future__ import annotations

from .._root import as_tensor, call_on_stream


def update_pix2tri(tri2vtx, vtx2xyz, bvhnodes, bvhnode2aabb, transform_ndc2world, pix2tri, stream_ptr=0):
    """Writes the closest-hit triangle of every pixel's ray into pix2tri
    (u32::MAX where nothing is hit).  Replaces pix2tri_by_raycast
    (del-msh-dlpack/src/pix2tri.rs:17-94)."""
    from .. import _native
    tri2vtx, vtx2xyz, bvhnodes, bvhnode2aabb, tf, pix2tri = map(
        as_tensor, (tri2vtx, vtx2xyz, bvhnodes, bvhnode2aabb, transform_ndc2world, pix2tri))
    img_h, img_w = pix2tri.shape[0], pix2tri.shape[1]
    num_tri, num_vtx = tri2vtx.shape[0], vtx2xyz.shape[0]
    nbytes = _native.load().dm_cast_scratch_bytes(img_w * img_h, num_tri)
    call_on_stream(stream_ptr, tri2vtx.device, nbytes, lambda scr: _native.call(
        "dm_pix2tri_by_raycast", stream_ptr, img_w, img_h, pix2tri.data_ptr(), None, num_tri, tri2vtx.data_ptr(),
        num_vtx, vtx2xyz.data_ptr(), bvhnodes.data_ptr(), bvhnode2aabb.data_ptr(), tf.data_ptr(),
        scr.data_ptr(), scr.numel()))


def interpolate(pix2tri, tri2vtx, vtx2xyz, vtx2val, transform_ndc2world, pix2val, stream_ptr=0):
    """pix2val[ih, iw, :] = vertex values interpolated at the pixel ray's hit
    (0 on the background).  Replaces pix2tri_interpolate."""
    from .. import _native
    pix2tri, tri2vtx, vtx2xyz, vtx2val, tf, pix2val = map(
        as_tensor, (pix2tri, tri2vtx, vtx2xyz, vtx2val, transform_ndc2world, pix2val))
    img_h, img_w = pix2tri.shape[0], pix2tri.shape[1]
    call_on_stream(stream_ptr, tri2vtx.device, 0, lambda _: _native.call(
        "dm_pix2tri_interpolate", stream_ptr, img_w, img_h, pix2tri.data_ptr(), tri2vtx.shape[0],
        tri2vtx.data_ptr(), vtx2xyz.shape[0], vtx2xyz.data_ptr(), vtx2val.shape[1], vtx2val.data_ptr(),
        tf.data_ptr(), pix2val.data_ptr()))


def interpolate_bwd(pix2tri, tri2vtx, vtx2xyz, vtx2val, transform_ndc2world, dldw_pix2val, dldw_vtx2xyz,
                    dldw_vtx2val, stream_ptr=0):
    """Adds the backward of ``interpolate`` into dldw_vtx2xyz and
    dldw_vtx2val.  Replaces pix2tri_interpolate_bwd."""
    from .. import _native
    pix2tri, tri2vtx, vtx2xyz, vtx2val, tf, g, gx, gv = map(
        as_tensor, (pix2tri, tri2vtx, vtx2xyz, vtx2val, transform_ndc2world, dldw_pix2val, dldw_vtx2xyz,
                    dldw_vtx2val))
    img_h, img_w = pix2tri.shape[0], pix2tri.shape[1]
    call_on_stream(stream_ptr, tri2vtx.device, 0, lambda _: _native.call(
        "dm_pix2tri_interpolate_bwd", stream_ptr, img_w, img_h, pix2tri.data_ptr(), tri2vtx.shape[0],
        tri2vtx.data_ptr(), vtx2xyz.shape[0], vtx2xyz.data_ptr(), vtx2val.shape[1], vtx2val.data_ptr(),
        tf.data_ptr(), g.data_ptr(), gx.data_ptr(), gv.data_ptr()))
