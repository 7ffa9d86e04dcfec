"""numpy front-end of the oracle (CPU restatement of del-msh-cpu's LBVH build
and BVH ray cast, ``oracle.c``) and of the reference's own Morton/topology code
compiled as host C++ (``oracle/_ref``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline / reference arm of ``bench.py``, always as what results
are tested against or as the timed CPU baseline — never by the product path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_lib = None
_ref = None
UMAX = 0xFFFFFFFF


def lib():
    global _lib
    if _lib is None:
        path = _build.LIB_ORACLE
        if not path.exists():
            _build.build_oracle()
        L = C.CDLL(str(path))
        u32, f32, i32, vp = C.c_uint32, C.c_float, C.c_int, C.c_void_p
        L.or_expand_bits3.restype = u32
        L.or_expand_bits3.argtypes = [u32]
        L.or_morton_code3.restype = u32
        L.or_morton_code3.argtypes = [f32, f32, f32]
        L.or_morton_code2.restype = u32
        L.or_morton_code2.argtypes = [f32, f32]
        L.or_tri2cntr.argtypes = [u32, _u32p, _f32p, _f32p]
        L.or_aabb3.argtypes = [u32, _f32p, _f32p]
        L.or_fit_into_unit_preserve_asp.argtypes = [_f32p, _f32p]
        L.or_vtx2morton.argtypes = [u32, u32, _f32p, _f32p, _u32p]
        L.or_argsort_stable.argtypes = [u32, _u32p, _u32p, _u32p]
        L.or_update_bvhnodes.argtypes = [u32, _u32p, _u32p, _u32p]
        L.or_bvhnodes_from_triangle_mesh.argtypes = [u32, _u32p, _f32p, _u32p, _f32p, _u32p, _u32p, _u32p]
        L.or_update_aabb_uniform_mesh.argtypes = [_f32p, u32, _u32p, _u32p, _f32p, vp]
        L.or_pix2tri_by_raycast.argtypes = [u32, u32, _f32p, _u32p, _f32p, _u32p, _f32p, _u32p, vp, i32]
        L.or_cast_rays.argtypes = [u32, _f32p, _f32p, _u32p, _f32p, _u32p, _f32p, _u32p, vp, i32]
        L.or_intersections_ray.restype = u32
        L.or_intersections_ray.argtypes = [_f32p, _f32p, _u32p, _f32p, _u32p, _f32p, _f32p, _u32p, u32]
        L.or_ray_for_pixel.argtypes = [u32, u32, u32, _f32p, _f32p, _f32p]
        L.or_tri3_ray_f64.restype = i32
        L.or_tri3_ray_f64.argtypes = [_f32p, _f32p, _f32p, _f32p, _f32p, C.POINTER(C.c_double)]
        L.or_check_bvh_topology.restype = i32
        L.or_check_bvh_topology.argtypes = [_u32p, u32]
        L.or_check_morton_code_range_split.restype = i32
        L.or_check_morton_code_range_split.argtypes = [_u32p, u32]
        L.or_tree_height.restype = u32
        L.or_tree_height.argtypes = [_u32p, u32]
        L.or_mat4_inverse_pivot.restype = i32
        L.or_mat4_inverse_pivot.argtypes = [_f32p, _f32p]
        L.or_pix2tri_by_rasterization.restype = i32
        L.or_pix2tri_by_rasterization.argtypes = [u32, u32, _f32p, u32, _u32p, _f32p, _u32p, _f32p]
        L.or_pix2depth.restype = i32
        L.or_pix2depth.argtypes = [u32, u32, _f32p, _u32p, u32, _u32p, u32, _f32p, _f32p]
        L.or_pix2depth_bwd.restype = i32
        L.or_pix2depth_bwd.argtypes = [u32, u32, _f32p, _u32p, u32, _u32p, u32, _f32p, _f32p, _f32p]
        L.or_interpolate.argtypes = [u32, u32, _u32p, u32, _u32p, u32, _f32p, u32, _f32p, _f32p, _f32p]
        L.or_qot_binary_radix_tree_and_depth.argtypes = [u32, _u32p, u32, u32, _u32p, _u32p]
        L.or_qot_bnode2onode_and_idx2bnode.argtypes = [u32, _u32p, _u32p, _u32p, _u32p]
        L.or_qot_make_tree.argtypes = [u32, _u32p, _u32p, _u32p, _u32p, _u32p, u32, u32, u32, _u32p, _u32p, _f32p,
                                       _u32p, _f32p]
        L.or_qot_aggregate.argtypes = [u32, u32, _f32p, _u32p, u32, _u32p, u32, _f32p]
        L.or_self_intersection.restype = u32
        L.or_self_intersection.argtypes = [_u32p, _f32p, _u32p, _f32p, u32, _u32p, _f32p]
        L.or_self_intersection_brute.restype = u32
        L.or_self_intersection_brute.argtypes = [u32, _u32p, _f32p, u32, _u32p, _f32p]
        L.or_qot_check.restype = i32
        L.or_qot_check.argtypes = [u32, u32, _u32p, _f32p, _u32p, _u32p, _f32p, u32, u32]
        L.or_interpolate_bwd.argtypes = [u32, u32, _u32p, u32, _u32p, u32, _f32p, u32, _f32p, _f32p, _f32p, _f32p,
                                         _f32p]
        L.or_pix2tri_work.argtypes = [u32, u32, _f32p, _u32p, _f32p, _u32p, _f32p,
                                      np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")]
        L.or_pix2tri_work_depth.restype = None
        L.or_pix2tri_work_depth.argtypes = [u32, u32, _f32p, _u32p, _f32p, _u32p, _f32p,
                                            np.ctypeslib.ndpointer(np.uint64, flags="C"),
                                            np.ctypeslib.ndpointer(np.uint64, flags="C"), u32]
        _lib = L
    return _lib


def ref_lib():
    """The reference's Morton/topology code compiled as host C++, or None when
    ``oracle/_ref`` was not built (no reference checkout on this machine)."""
    global _ref
    if _ref is None:
        path = _build.LIB_REF
        if not path.exists():
            if _build.build_ref() is None:
                return None
        L = C.CDLL(str(path))
        u32, f32 = C.c_uint32, C.c_float
        L.ref_expand_bits3.restype = u32
        L.ref_expand_bits3.argtypes = [u32]
        L.ref_morton_code3.restype = u32
        L.ref_morton_code3.argtypes = [f32, f32, f32]
        L.ref_morton_code2.restype = u32
        L.ref_morton_code2.argtypes = [f32, f32]
        L.ref_bvh_topology.argtypes = [u32, _u32p, _u32p, _u32p]
        L.ref_tri2cntr.argtypes = [u32, _u32p, _f32p, _f32p]
        _ref = L
    return _ref


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def _vp(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def default_threads() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


# ----------------------------------------------------------------- build

def tri2cntr(tri2vtx, vtx2xyz):
    tri2vtx, vtx2xyz = _c(tri2vtx, np.uint32), _c(vtx2xyz, np.float32)
    out = np.empty((tri2vtx.size // 3, 3), np.float32)
    lib().or_tri2cntr(tri2vtx.size // 3, tri2vtx.reshape(-1), vtx2xyz.reshape(-1), out.reshape(-1))
    return out


def aabb3(pnt2xyz):
    p = _c(pnt2xyz, np.float32)
    out = np.empty(6, np.float32)
    lib().or_aabb3(p.size // 3, p.reshape(-1), out)
    return out


def fit_into_unit_preserve_asp(aabb):
    out = np.empty(16, np.float32)
    lib().or_fit_into_unit_preserve_asp(_c(aabb, np.float32), out)
    return out


def vtx2morton(vtx2co, transform_colmajor):
    v = _c(vtx2co, np.float32)
    n, dim = v.shape
    out = np.empty(n, np.uint32)
    lib().or_vtx2morton(n, dim, v.reshape(-1), _c(transform_colmajor, np.float32).reshape(-1), out)
    return out


def argsort_stable(codes):
    codes = _c(codes, np.uint32)
    idx = np.empty_like(codes)
    srt = np.empty_like(codes)
    lib().or_argsort_stable(codes.size, codes, idx, srt)
    return idx, srt


def update_bvhnodes(idx2obj, idx2morton):
    idx2obj, idx2morton = _c(idx2obj, np.uint32), _c(idx2morton, np.uint32)
    n = idx2obj.size
    out = np.zeros((2 * n - 1, 3), np.uint32)
    lib().or_update_bvhnodes(n, idx2obj, idx2morton, out.reshape(-1))
    return out


def bvhnodes_from_triangle_mesh(tri2vtx, vtx2xyz):
    """Returns dict(bvhnodes, transform, tri2morton, idx2tri, idx2morton)."""
    tri2vtx, vtx2xyz = _c(tri2vtx, np.uint32), _c(vtx2xyz, np.float32)
    T = tri2vtx.size // 3
    bvh = np.zeros((2 * T - 1, 3), np.uint32)
    m = np.empty(16, np.float32)
    t2m = np.empty(T, np.uint32)
    i2t = np.empty(T, np.uint32)
    i2m = np.empty(T, np.uint32)
    lib().or_bvhnodes_from_triangle_mesh(T, tri2vtx.reshape(-1), vtx2xyz.reshape(-1), bvh.reshape(-1), m, t2m,
                                         i2t, i2m)
    return dict(bvhnodes=bvh, transform=m, tri2morton=t2m, idx2tri=i2t, idx2morton=i2m)


def bvhnode2aabb(bvhnodes, tri2vtx, vtx2xyz, vtx2xyz1=None):
    bvhnodes, tri2vtx, vtx2xyz = _c(bvhnodes, np.uint32), _c(tri2vtx, np.uint32), _c(vtx2xyz, np.float32)
    out = np.zeros((bvhnodes.size // 3, 6), np.float32)
    v1 = None if vtx2xyz1 is None else _c(vtx2xyz1, np.float32)
    lib().or_update_aabb_uniform_mesh(out.reshape(-1), 0, bvhnodes.reshape(-1), tri2vtx.reshape(-1),
                                      vtx2xyz.reshape(-1), _vp(v1))
    return out


def build(tri2vtx, vtx2xyz):
    r = bvhnodes_from_triangle_mesh(tri2vtx, vtx2xyz)
    r["bvhnode2aabb"] = bvhnode2aabb(r["bvhnodes"], tri2vtx, vtx2xyz)
    return r


# ------------------------------------------------------------------ cast

def pix2tri(tri2vtx, vtx2xyz, bvhnodes, aabb, t_ndc2world_colmajor, img_w, img_h, threads=None, want_t=True):
    tri2vtx, vtx2xyz = _c(tri2vtx, np.uint32), _c(vtx2xyz, np.float32)
    bvhnodes, aabb = _c(bvhnodes, np.uint32), _c(aabb, np.float32)
    out = np.empty((img_h, img_w), np.uint32)
    tt = np.empty((img_h, img_w), np.float32) if want_t else None
    lib().or_pix2tri_by_raycast(img_w, img_h, _c(t_ndc2world_colmajor, np.float32).reshape(-1),
                                tri2vtx.reshape(-1), vtx2xyz.reshape(-1), bvhnodes.reshape(-1), aabb.reshape(-1),
                                out.reshape(-1), _vp(tt), threads or default_threads())
    return out, tt


def pix2tri_work(tri2vtx, vtx2xyz, bvhnodes, aabb, t_ndc2world_colmajor, img_w, img_h):
    """The recursion's work over a pixel grid: rays, branches entered (two child
    boxes tested each) and triangles tested, counted on one thread."""
    out = np.zeros(3, np.uint64)
    lib().or_pix2tri_work(img_w, img_h, _c(t_ndc2world_colmajor, np.float32).reshape(-1),
                          _c(tri2vtx, np.uint32).reshape(-1), _c(vtx2xyz, np.float32).reshape(-1),
                          _c(bvhnodes, np.uint32).reshape(-1), _c(aabb, np.float32).reshape(-1), out)
    return {"rays": int(out[0]), "branches": int(out[1]), "tri_tests": int(out[2])}


def pix2tri_work_depth(tri2vtx, vtx2xyz, bvhnodes, aabb, t_ndc2world_colmajor, img_w, img_h, max_depth=64):
    """pix2tri_work's counts and the branches entered per tree depth (root 0;
    the last bin takes every deeper entry)."""
    out = np.zeros(3, np.uint64)
    hist = np.zeros(max_depth, np.uint64)
    lib().or_pix2tri_work_depth(img_w, img_h, _c(t_ndc2world_colmajor, np.float32).reshape(-1),
                                _c(tri2vtx, np.uint32).reshape(-1), _c(vtx2xyz, np.float32).reshape(-1),
                                _c(bvhnodes, np.uint32).reshape(-1), _c(aabb, np.float32).reshape(-1), out, hist,
                                max_depth)
    return out, hist


def cast_rays(ray_org, ray_dir, tri2vtx, vtx2xyz, bvhnodes, aabb, threads=None):
    ro, rd = _c(ray_org, np.float32), _c(ray_dir, np.float32)
    n = ro.size // 3
    hit = np.empty(n, np.uint32)
    t = np.empty(n, np.float32)
    lib().or_cast_rays(n, ro.reshape(-1), rd.reshape(-1), _c(tri2vtx, np.uint32).reshape(-1),
                       _c(vtx2xyz, np.float32).reshape(-1), _c(bvhnodes, np.uint32).reshape(-1),
                       _c(aabb, np.float32).reshape(-1), hit, _vp(t), threads or default_threads())
    return hit, t


def intersections_ray(org, dir, tri2vtx, vtx2xyz, bvhnodes, aabb, cap=64):
    ht = np.empty(cap, np.float32)
    hi = np.empty(cap, np.uint32)
    n = lib().or_intersections_ray(_c(org, np.float32), _c(dir, np.float32), _c(tri2vtx, np.uint32).reshape(-1),
                                   _c(vtx2xyz, np.float32).reshape(-1), _c(bvhnodes, np.uint32).reshape(-1),
                                   _c(aabb, np.float32).reshape(-1), ht, hi, cap)
    return ht[:min(n, cap)], hi[:min(n, cap)], n


def ray_for_pixel(i_pix, img_w, img_h, t_ndc2world_colmajor):
    org = np.empty(3, np.float32)
    d = np.empty(3, np.float32)
    lib().or_ray_for_pixel(i_pix, img_w, img_h, _c(t_ndc2world_colmajor, np.float32).reshape(-1), org, d)
    return org, d


def tri3_ray_f64(p0, p1, p2, org, dir):
    t = C.c_double(0.0)
    ok = lib().or_tri3_ray_f64(_c(p0, np.float32), _c(p1, np.float32), _c(p2, np.float32), _c(org, np.float32),
                               _c(dir, np.float32), C.byref(t))
    return t.value if ok else None


def check_bvh_topology(bvhnodes, num_leaf):
    return bool(lib().or_check_bvh_topology(_c(bvhnodes, np.uint32).reshape(-1), num_leaf))


def check_morton_code_range_split(idx2morton):
    c = _c(idx2morton, np.uint32)
    return bool(lib().or_check_morton_code_range_split(c, c.size))


def tree_height(bvhnodes, num_leaf):
    return int(lib().or_tree_height(_c(bvhnodes, np.uint32).reshape(-1), num_leaf))


# ------------------------------------- consumers of a pix2tri image

def pix2tri_by_rasterization(tri2vtx, vtx2xyz, t_ndc2world_colmajor, img_w, img_h):
    """(pix2tri, pix2depth) of pix2tri.rs:50-119 (u32::MAX / -inf where nothing covers)."""
    tri2vtx, vtx2xyz = _c(tri2vtx, np.uint32), _c(vtx2xyz, np.float32)
    out = np.empty((img_h, img_w), np.uint32)
    depth = np.empty((img_h, img_w), np.float32)
    ok = lib().or_pix2tri_by_rasterization(img_w, img_h, _c(t_ndc2world_colmajor, np.float32).reshape(-1),
                                           tri2vtx.size // 3, tri2vtx.reshape(-1), vtx2xyz.reshape(-1), out, depth)
    if not ok:
        raise ValueError("transform_ndc2world is singular")
    return out, depth


def mat4_inverse_pivot(m_colmajor):
    inv = np.empty(16, np.float32)
    ok = lib().or_mat4_inverse_pivot(_c(m_colmajor, np.float32).reshape(-1), inv)
    return inv, bool(ok)


def pix2depth(pix2tri, tri2vtx, vtx2xyz, t_ndc2world_colmajor, img_w, img_h, init=None):
    """pix2depth.rs:107-146 restated; pixels whose ray misses their triangle
    keep `init` (zeros by default)."""
    out = np.zeros(img_w * img_h, np.float32) if init is None else _c(init, np.float32).reshape(-1).copy()
    tri2vtx, vtx2xyz = _c(tri2vtx, np.uint32), _c(vtx2xyz, np.float32)
    lib().or_pix2depth(img_w, img_h, out, _c(pix2tri, np.uint32).reshape(-1), tri2vtx.size // 3, tri2vtx.reshape(-1),
                       vtx2xyz.size // 3, vtx2xyz.reshape(-1), _c(t_ndc2world_colmajor, np.float32).reshape(-1))
    return out.reshape(img_h, img_w)


def pix2depth_bwd(pix2tri, tri2vtx, vtx2xyz, dldw_pix2depth, t_ndc2world_colmajor, img_w, img_h, init=None):
    tri2vtx, vtx2xyz = _c(tri2vtx, np.uint32), _c(vtx2xyz, np.float32)
    g = np.zeros(vtx2xyz.size, np.float32) if init is None else _c(init, np.float32).reshape(-1).copy()
    lib().or_pix2depth_bwd(img_w, img_h, g, _c(pix2tri, np.uint32).reshape(-1), tri2vtx.size // 3,
                           tri2vtx.reshape(-1), vtx2xyz.size // 3, vtx2xyz.reshape(-1),
                           _c(dldw_pix2depth, np.float32).reshape(-1), _c(t_ndc2world_colmajor, np.float32).reshape(-1))
    return g.reshape(-1, 3)


def interpolate(pix2tri, tri2vtx, vtx2xyz, vtx2val, t_ndc2world_colmajor, img_w, img_h):
    tri2vtx, vtx2xyz, vtx2val = _c(tri2vtx, np.uint32), _c(vtx2xyz, np.float32), _c(vtx2val, np.float32)
    nd = vtx2val.shape[1]
    out = np.empty(img_w * img_h * nd, np.float32)
    lib().or_interpolate(img_w, img_h, _c(pix2tri, np.uint32).reshape(-1), tri2vtx.size // 3, tri2vtx.reshape(-1),
                         vtx2xyz.size // 3, vtx2xyz.reshape(-1), nd, vtx2val.reshape(-1),
                         _c(t_ndc2world_colmajor, np.float32).reshape(-1), out)
    return out.reshape(img_h, img_w, nd)


def interpolate_bwd(pix2tri, tri2vtx, vtx2xyz, vtx2val, t_ndc2world_colmajor, dldw_pix2val, img_w, img_h):
    tri2vtx, vtx2xyz, vtx2val = _c(tri2vtx, np.uint32), _c(vtx2xyz, np.float32), _c(vtx2val, np.float32)
    nd = vtx2val.shape[1]
    gx = np.zeros(vtx2xyz.size, np.float32)
    gv = np.zeros(vtx2val.size, np.float32)
    lib().or_interpolate_bwd(img_w, img_h, _c(pix2tri, np.uint32).reshape(-1), tri2vtx.size // 3, tri2vtx.reshape(-1),
                             vtx2xyz.size // 3, vtx2xyz.reshape(-1), nd, vtx2val.reshape(-1),
                             _c(t_ndc2world_colmajor, np.float32).reshape(-1),
                             _c(dldw_pix2val, np.float32).reshape(-1), gx, gv)
    return gx.reshape(-1, 3), gv.reshape(-1, nd)


# ---------------------------------------------------------- quad/oct-trees

def quad_oct_tree(idx2morton, num_dim, max_depth=None):
    """quad_oct_tree.rs restated: binary radix tree, bnode2onode, idx2bnode
    and the quad/oct-tree of sorted unique codes; returns a dict."""
    c = _c(idx2morton, np.uint32).reshape(-1)
    max_depth = 32 // num_dim if max_depth is None else max_depth
    n = c.size
    bnodes = np.zeros((n - 1) * 3, np.uint32)
    b2d = np.zeros(n - 1, np.uint32)
    lib().or_qot_binary_radix_tree_and_depth(n, c, num_dim, max_depth, bnodes, b2d)
    b2o = np.zeros(n - 1, np.uint32)
    i2b = np.full(n, 0xFFFFFFFF, np.uint32)
    lib().or_qot_bnode2onode_and_idx2bnode(n, bnodes, b2d, b2o, i2b)
    num_onode = int(b2o[-1]) + 1
    nlink = 1 + 2 ** num_dim
    onodes = np.full(num_onode * nlink, 0xFFFFFFFF, np.uint32)
    o2d = np.zeros(num_onode, np.uint32)
    o2c = np.zeros(num_onode * num_dim, np.float32)
    i2o = np.zeros(n, np.uint32)
    i2c = np.zeros(n * num_dim, np.float32)
    lib().or_qot_make_tree(n, bnodes, b2o, b2d, i2b, c, num_onode, max_depth, num_dim, onodes, o2d, o2c, i2o, i2c)
    return dict(bnodes=bnodes.reshape(-1, 3), bnode2depth=b2d, bnode2onode=b2o, idx2bnode=i2b, num_onode=num_onode,
                onodes=onodes.reshape(num_onode, nlink), onode2depth=o2d, onode2center=o2c.reshape(-1, num_dim),
                idx2onode=i2o, idx2center=i2c.reshape(-1, num_dim), max_depth=max_depth)


def quad_oct_tree_check(t, num_dim):
    return bool(lib().or_qot_check(t["idx2onode"].size, num_dim, t["idx2onode"], _c(t["idx2center"], np.float32),
                                   _c(t["onodes"], np.uint32), t["onode2depth"], _c(t["onode2center"], np.float32),
                                   t["num_onode"], t["max_depth"]))


def quad_oct_tree_aggregate(idx2val, idx2onode, onodes):
    v = _c(idx2val, np.float32)
    nd = v.shape[1]
    on = _c(onodes, np.uint32)
    out = np.zeros(on.shape[0] * nd, np.float32)
    lib().or_qot_aggregate(v.shape[0], nd, v.reshape(-1), _c(idx2onode, np.uint32), on.shape[1], on.reshape(-1),
                           on.shape[0], out)
    return out.reshape(-1, nd)


# ------------------------------------------------------- self-intersection

def self_intersection(tri2vtx, vtx2xyz, bvhnodes, aabb, brute=False):
    """trimesh3_intersection.rs restated: (pairs u32[k][2], segments f32[k][6])
    in the reference's visiting order (BVH search), or i < j order (brute)."""
    tri2vtx, vtx2xyz = _c(tri2vtx, np.uint32), _c(vtx2xyz, np.float32)
    cap = 1 << 16
    while True:
        pairs = np.zeros(cap * 2, np.uint32)
        segs = np.zeros(cap * 6, np.float32)
        if brute:
            n = lib().or_self_intersection_brute(tri2vtx.size // 3, tri2vtx.reshape(-1), vtx2xyz.reshape(-1), cap,
                                                 pairs, segs)
        else:
            n = lib().or_self_intersection(tri2vtx.reshape(-1), vtx2xyz.reshape(-1),
                                           _c(bvhnodes, np.uint32).reshape(-1), _c(aabb, np.float32).reshape(-1),
                                           cap, pairs, segs)
        if n <= cap:
            return pairs[: 2 * n].reshape(-1, 2), segs[: 6 * n].reshape(-1, 6)
        cap = n


# ---------------------------------------------------------- reference code

def ref_bvh_topology(idx2morton, idx2obj):
    """The reference's kernel_MortonCode_BVHTopology run on the host."""
    L = ref_lib()
    if L is None:
        return None
    idx2morton, idx2obj = _c(idx2morton, np.uint32), _c(idx2obj, np.uint32)
    n = idx2obj.size
    out = np.zeros((2 * n - 1, 3), np.uint32)
    L.ref_bvh_topology(n, idx2morton, idx2obj, out.reshape(-1))
    return out


def ref_tri2cntr(tri2vtx, vtx2xyz):
    L = ref_lib()
    if L is None:
        return None
    tri2vtx, vtx2xyz = _c(tri2vtx, np.uint32), _c(vtx2xyz, np.float32)
    out = np.empty((tri2vtx.size // 3, 3), np.float32)
    L.ref_tri2cntr(tri2vtx.size // 3, tri2vtx.reshape(-1), vtx2xyz.reshape(-1), out.reshape(-1))
    return out
