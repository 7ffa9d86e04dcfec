"""The reference's pixel-level pin of the ray cast (del-msh-cpu
pix2tri.rs:121-173): on a 256x256 image of a rotated and translated torus,
the triangle hit by each pixel's ray equals the triangle the rasteriser
(pix2tri.rs:50-119) puts there, for every pixel.  Here on the oracle; the
GPU cast is held to the same rasterised image in test_gpu_cast.py."""
import numpy as np

from helpers import reference_pin_torus

UMAX = 0xFFFFFFFF


def test_rasteriser_covers_pixel_centres(oracle):
    # one triangle over pixel space (ndc2world = identity): x in [-1, 1] -> [0, 8)
    tri = np.array([[0, 1, 2]], np.uint32)
    vtx = np.array([[-1, 1, 0], [1, 1, 0], [-1, -1, 0]], np.float32)  # upper-left half
    p2t, depth = oracle.pix2tri_by_rasterization(tri, vtx, np.eye(4, dtype=np.float32).reshape(-1), 8, 8)
    # centre (ix + .5, iy + .5) is covered iff ix + iy <= 7 (on or above the diagonal)
    iy, ix = np.mgrid[0:8, 0:8]
    assert np.array_equal(p2t == 0, ix + iy <= 7)
    assert np.isneginf(depth[p2t == UMAX]).all()


def test_raycast_equals_rasterisation_every_pixel(oracle):
    tri, vtx, m = reference_pin_torus()
    r = oracle.build(tri, vtx)
    ray, _ = oracle.pix2tri(tri, vtx, r["bvhnodes"], r["bvhnode2aabb"], m, 256, 256)
    ras, _ = oracle.pix2tri_by_rasterization(tri, vtx, m, 256, 256)
    assert (ray != UMAX).sum() > 10000
    assert np.array_equal(ray, ras)
