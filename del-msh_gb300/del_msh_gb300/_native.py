"""ctypes binding of ``libdelmsh_gb300.so`` (the C ABI in include/delmsh_gb300.h).

There is no CPU fallback: if the library is missing or cannot be loaded the
first call raises, naming the build step to run.
"""
from __future__ import annotations

import ctypes as C
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

u32, u64, f32p, u32p, vp, sz, i32 = C.c_uint32, C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_int

_SIGNATURES = {
    "dm_version": (C.c_char_p, []),
    "dm_last_error": (C.c_char_p, []),
    "dm_device_status": (i32, [C.POINTER(C.c_uint32), i32]),
    "dm_tuning_get": (i32, [vp]),
    "dm_render_scratch_bytes": (sz, []),
    "dm_trimesh3_self_intersection": (i32, [u64, u32, vp, u32, vp, vp, vp, u32, vp, vp, vp]),
    "dm_quad_oct_tree_scratch_bytes": (sz, [u32]),
    "dm_quad_oct_tree_bnodes_and_bnode2depth_and_bnode2onode_and_idx2bnode":
        (i32, [u64, u32, vp, u32, u32, vp, vp, vp, vp, vp, sz]),
    "dm_quad_oct_tree_make_tree_from_binary_radix_tree":
        (i32, [u64, u32, vp, vp, vp, vp, vp, u32, u32, u32, vp, vp, vp, vp, vp]),
    "dm_quad_oct_tree_aggregate": (i32, [u64, u32, u32, vp, vp, u32, vp, u32, vp]),
    "dm_pix2depth_update": (i32, [u64, u32, u32, vp, vp, u32, vp, u32, vp, vp, vp, sz]),
    "dm_pix2depth_bwd_wrt_vtx2xyz": (i32, [u64, u32, u32, vp, vp, u32, vp, u32, vp, vp, vp, vp, sz]),
    "dm_pix2tri_interpolate": (i32, [u64, u32, u32, vp, u32, vp, u32, vp, u32, vp, vp, vp]),
    "dm_pix2tri_interpolate_bwd": (i32, [u64, u32, u32, vp, u32, vp, u32, vp, u32, vp, vp, vp, vp, vp]),
    "dm_tuning_set": (i32, [vp]),
    "dm_build_classes_set": (i32, [vp, u32]),
    "dm_build_classes_get": (i32, [vp, u32, vp]),
    "dm_wait_limit_get": (i32, [vp]),
    "dm_wait_limit_set": (i32, [u32]),
    "dm_selftest_bounded_wait": (i32, [u64, u32, vp, sz]),
    "dm_selftest_bounded_wait_scratch_bytes": (sz, []),
    "dm_mortons_vtx2morton_from_vtx2co": (i32, [u64, u32, u32, vp, vp, vp]),
    "dm_array1d_argsort": (i32, [u64, u32, vp, vp, vp, sz]),
    "dm_array1d_argsort_scratch_bytes": (sz, [u32]),
    "dm_mortons_make_bvhnodes_from_sorted_mortons": (i32, [u64, u32, vp, vp, vp]),
    "dm_bvhnode2aabb_update_aabb": (i32, [u64, u32, vp, u32, vp, u32, vp, u32, vp, vp, vp]),
    "dm_bvhnode2aabb_update_aabb_noalloc": (i32, [u64, u32, vp, vp, u32, vp, u32, vp, vp]),
    "dm_bvhnode2aabb_update_aabb_ex": (i32, [u64, u32, vp, vp, u32, vp, u32, vp, vp, vp, sz]),
    "dm_bvhnode2aabb_update_aabb_scratch_bytes": (sz, [u32]),
    "dm_trimesh3_make_bvhnodes_bvhnode2aabb": (i32, [u64, u32, vp, u32, vp, vp, vp, vp, sz]),
    "dm_trimesh3_build_scratch_bytes": (sz, [u32]),
    "dm_trimesh3_build_ex": (i32, [u64, u32, vp, u32, vp, vp, vp, vp, vp, vp, vp, vp, vp, sz]),
    "dm_trimesh3_build_profiled": (i32, [u64, u32, vp, u32, vp, vp, vp, vp, sz, vp]),
    "dm_pix2tri_by_raycast": (i32, [u64, u32, u32, vp, vp, u32, vp, u32, vp, vp, vp, vp, vp, sz]),
    "dm_search_bvh3_first_intersection_ray": (i32, [u64, u32, vp, vp, vp, vp, vp, u32, vp, u32, vp, vp, vp, vp, sz]),
    "dm_cast_scratch_bytes": (sz, [u32, u32]),
    "dm_batch_trimesh3_build": (i32, [u64, u32, vp, vp, u32, u32, u32, vp, vp, vp, vp, vp, vp, sz]),
    "dm_batch_build_scratch_bytes": (sz, [u32, u32]),
    "dm_batch_pix2tri_by_raycast": (i32, [u64, u32, vp, vp, u32, u32, u32, vp, vp, vp, vp, u32, u32, vp, vp, vp, vp,
                                          sz]),
    "dm_batch_cast_scratch_bytes": (sz, [u32, u32]),
}

# request-server entry points; their ctypes signatures (with the request /
# result structures) are set by del_msh_gb300.serve
SERVER_FUNCS = ("dm_server_create", "dm_server_register_mesh", "dm_server_submit", "dm_server_wait",
                "dm_server_run_trace", "dm_plain_run_trace", "dm_server_stats_get", "dm_server_destroy")

# entry points that return a status code
STATUS_FUNCS = {k for k, (r, _) in _SIGNATURES.items() if r is i32 and k != "dm_device_status"}


class Tuning(C.Structure):
    """dm_tuning of include/delmsh_gb300.h."""
    _fields_ = [("cast_threads", C.c_uint32), ("cast_stack", C.c_uint32), ("tile_w", C.c_uint32),
                ("sort_window", C.c_uint32), ("cast_refill_min", C.c_uint32), ("cast_leaf_min", C.c_uint32),
                ("cast_ascend_min", C.c_uint32), ("cast_long_steps", C.c_uint32), ("batch_path", C.c_uint32),
                ("batch_cluster", C.c_uint32)]
    KEYS = ("cast_threads", "cast_stack", "tile_w", "sort_window", "cast_refill_min", "cast_leaf_min",
            "cast_ascend_min", "cast_long_steps", "batch_path", "batch_cluster")

    def as_dict(self):
        return {k: int(getattr(self, k)) for k in self.KEYS}


class BuildClass(C.Structure):
    """dm_build_class of include/delmsh_gb300.h."""
    _fields_ = [("max_tri", C.c_uint32), ("build_path", C.c_uint32), ("sort_radix", C.c_uint32),
                ("topo_threads", C.c_uint32)]
    KEYS = ("max_tri", "build_path", "sort_radix", "topo_threads")


def set_build_classes(classes) -> None:
    """Sets the single-mesh build's size classes (a list of dicts with the
    BuildClass keys, bounds ascending; [] clears them)."""
    arr = (BuildClass * max(1, len(classes)))(*[BuildClass(*(int(c.get(k, 0)) for k in BuildClass.KEYS))
                                                 for c in classes])
    call("dm_build_classes_set", C.addressof(arr), len(classes))


def get_build_classes() -> list:
    arr = (BuildClass * 8)()
    n = C.c_uint32(0)
    call("dm_build_classes_get", C.addressof(arr), 8, C.byref(n))
    return [{k: int(getattr(arr[i], k)) for k in BuildClass.KEYS} for i in range(n.value)]


def get_tuning() -> dict:
    t = Tuning()
    call("dm_tuning_get", C.addressof(t))
    return t.as_dict()


def set_tuning(cast_threads: int, cast_stack: int, tile_w: int, sort_window: int, cast_refill_min: int = 0,
               cast_leaf_min: int = 0, cast_ascend_min: int = 0, cast_long_steps: int = 0, batch_path: int = 0,
               batch_cluster: int = 0) -> None:
    """Sets dm_tuning; a phase minimum or step budget of 0 selects the library default."""
    t = Tuning(cast_threads, cast_stack, tile_w, sort_window, cast_refill_min, cast_leaf_min, cast_ascend_min,
               cast_long_steps, batch_path, batch_cluster)
    call("dm_tuning_set", C.addressof(t))


def get_wait_limit() -> int:
    v = C.c_uint32(0)
    call("dm_wait_limit_get", C.byref(v))
    return int(v.value)


def set_wait_limit(polls: int) -> None:
    """Polls a bounded device wait makes before giving up (0 = the default)."""
    call("dm_wait_limit_set", polls)


class DelMshError(RuntimeError):
    """A non-zero status returned by the C ABI."""

    def __init__(self, func: str, code: int, message: str):
        super().__init__(f"{func} failed with status {code}: {message}")
        self.code = code


def lib_path():
    return _build.LIB_PATH


def load(build_if_missing: bool = False):
    """Loads the library; with build_if_missing it first compiles it."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB_PATH
        if not path.exists():
            if build_if_missing:
                _build.build()
            else:
                raise RuntimeError(f"{path} is missing: build it with `python -c \"import __graft_entry__ as g; "
                                   f"g.build()\"` (or del_msh_gb300.build.build()); there is no CPU fallback")
        L = C.CDLL(str(path))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    # the autotuned launch parameters for this device model, if a table was made
    try:
        from . import autotune
        autotune.apply()
    except Exception:  # a malformed or foreign table leaves the defaults
        pass
    return L


def exported_symbols():
    return sorted(set(_SIGNATURES) | set(SERVER_FUNCS))


def call(name: str, *args):
    """Calls a status-returning entry point and raises DelMshError on failure."""
    L = load()
    rc = getattr(L, name)(*args)
    if rc != 0:
        raise DelMshError(name, rc, L.dm_last_error().decode())
    return rc


def device_status(clear: bool = True) -> int:
    L = load()
    bits = C.c_uint32(0)
    rc = L.dm_device_status(C.byref(bits), 1 if clear else 0)
    if rc != 0:
        raise DelMshError("dm_device_status", rc, L.dm_last_error().decode())
    return bits.value
