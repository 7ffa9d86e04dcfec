"""Python driver of the request server (``dm_server_*`` in the C ABI).

``Server`` registers meshes and runs open-loop request traces through the
server (``run_trace``) or the plain serial path (``run_plain``);
``served_workload`` builds the seeded request stream of the served
configuration: a pool of icospheres / tori with log-uniform triangle counts,
Poisson arrivals, and a 20/60/20 mix of build+cast (512x512 pixels),
refit+re-cast after a per-frame deformation of a resident tree, and cast-only
requests of random rays.  No reference counterpart: del-msh has no server.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _native, workloads

BUILD_CAST, REFIT_CAST, CAST_RAYS = 0, 1, 2


class Request(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("mesh_id", C.c_uint32), ("frame", C.c_uint32), ("deform_amplitude", C.c_float),
                ("img_w", C.c_uint32), ("img_h", C.c_uint32), ("num_ray", C.c_uint32), ("reserved", C.c_uint32),
                ("transform_ndc2world", C.c_void_p), ("ray_org", C.c_void_p), ("ray_dir", C.c_void_p),
                ("out_tri", C.c_void_p), ("out_t", C.c_void_p)]


class Result(C.Structure):
    _fields_ = [("status", C.c_int32), ("resident_hit", C.c_uint32), ("t_submit_ns", C.c_uint64),
                ("t_admit_ns", C.c_uint64), ("t_done_ns", C.c_uint64)]


class Stats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("resident_hits", C.c_uint64),
                ("builds", C.c_uint64), ("refits", C.c_uint64), ("evictions", C.c_uint64),
                ("bytes_resident", C.c_uint64), ("bytes_budget", C.c_uint64), ("bytes_slots", C.c_uint64),
                ("meshes_resident", C.c_uint32),
                ("reserved", C.c_uint32)]


def _bind(L):
    if getattr(L, "_serve_bound", False):
        return
    vp, u32, i32, sz = C.c_void_p, C.c_uint32, C.c_int, C.c_size_t
    L.dm_server_create.argtypes = [i32, sz, i32, u32, u32, C.POINTER(vp)]
    L.dm_server_register_mesh.argtypes = [vp, u32, vp, u32, vp, u32, u32]
    L.dm_server_submit.argtypes = [vp, C.POINTER(Request), C.POINTER(C.c_uint64)]
    L.dm_server_wait.argtypes = [vp, C.c_uint64, C.POINTER(Result)]
    L.dm_server_run_trace.argtypes = [vp, u32, C.POINTER(Request), C.POINTER(C.c_double), C.POINTER(Result)]
    L.dm_plain_run_trace.argtypes = [vp, u32, C.POINTER(Request), C.POINTER(C.c_double), C.POINTER(Result)]
    L.dm_server_stats_get.argtypes = [vp, C.POINTER(Stats)]
    L.dm_server_destroy.argtypes = [vp]
    for f in _native.SERVER_FUNCS:
        getattr(L, f).restype = i32
    L._serve_bound = True


def _check(L, name, rc):
    if rc != 0:
        raise _native.DelMshError(name, rc, L.dm_last_error().decode())


def pinned(shape, dtype):
    """A numpy view of pinned host memory (kept alive by the returned tensor)."""
    tdt = {np.uint32: torch.int32, np.float32: torch.float32}[dtype]
    t = torch.empty(shape, dtype=tdt).pin_memory()
    return t, t.numpy().view(dtype)


class Server:
    def __init__(self, budget_bytes: int, num_slots: int, max_tri: int, max_out: int, device: int = 0):
        self.L = _native.load()
        _bind(self.L)
        h = C.c_void_p()
        _check(self.L, "dm_server_create",
               self.L.dm_server_create(device, budget_bytes, num_slots, max_tri, max_out, C.byref(h)))
        self.h = h
        self._keep = []

    def register(self, mesh_id: int, tri2vtx: np.ndarray, vtx2xyz: np.ndarray, seed: int):
        tri = np.ascontiguousarray(tri2vtx, np.uint32)
        vtx = np.ascontiguousarray(vtx2xyz, np.float32)
        _check(self.L, "dm_server_register_mesh",
               self.L.dm_server_register_mesh(self.h, mesh_id, tri.ctypes.data, tri.shape[0], vtx.ctypes.data,
                                              vtx.shape[0], seed))

    def _trace(self, fn, reqs, arrivals):
        n = len(reqs)
        arr = (Request * n)(*reqs)
        at = (C.c_double * n)(*[float(a) for a in arrivals])
        res = (Result * n)()
        _check(self.L, fn, getattr(self.L, fn)(self.h, n, arr, at, res))
        return res

    def run_trace(self, reqs, arrivals):
        return self._trace("dm_server_run_trace", reqs, arrivals)

    def run_plain(self, reqs, arrivals):
        return self._trace("dm_plain_run_trace", reqs, arrivals)

    def submit_and_wait(self, req: Request) -> Result:
        t = C.c_uint64()
        _check(self.L, "dm_server_submit", self.L.dm_server_submit(self.h, C.byref(req), C.byref(t)))
        r = Result()
        _check(self.L, "dm_server_wait", self.L.dm_server_wait(self.h, t.value, C.byref(r)))
        return r

    def stats(self) -> dict:
        s = Stats()
        _check(self.L, "dm_server_stats_get", self.L.dm_server_stats_get(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in Stats._fields_ if k != "reserved"}

    def close(self):
        if self.h:
            self.L.dm_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def latency_stats(results, t_scale=1e-6, kinds=None):
    """p50 / p99 / mean latency in ms (done - scheduled arrival) and the span;
    with `kinds` (the request kind of each result) also, per kind, the count,
    p50 / p99 latency and the mean wait before admission."""
    lat = np.array([(r.t_done_ns - r.t_submit_ns) for r in results], np.float64) * t_scale
    wait = np.array([(r.t_admit_ns - r.t_submit_ns) for r in results], np.float64) * t_scale
    t0 = min(r.t_submit_ns for r in results)
    t1 = max(r.t_done_ns for r in results)
    ok = all(r.status == 0 for r in results)
    out = {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
           "mean_ms": float(lat.mean()), "span_s": (t1 - t0) * 1e-9, "all_ok": ok}
    if kinds is not None:
        kinds = np.asarray(kinds)
        out["by_kind"] = {name: {"n": int((kinds == k).sum()),
                                 "p50_ms": float(np.percentile(lat[kinds == k], 50)),
                                 "p99_ms": float(np.percentile(lat[kinds == k], 99)),
                                 "mean_wait_ms": float(wait[kinds == k].mean())}
                          for k, name in ((BUILD_CAST, "build_cast"), (REFIT_CAST, "refit_cast"),
                                          (CAST_RAYS, "cast_rays")) if (kinds == k).any()}
    return out


class ServedWorkload:
    """The served configuration: pool, cameras, ray sets and a request stream."""

    def __init__(self, num_mesh=512, tmin=1000, tmax=1_000_000, img=512, num_ray=16384, seed=0,
                 mix=(0.2, 0.6, 0.2), amplitude=0.01, ring=64):
        self.meshes = workloads.ragged_batch(num_mesh=num_mesh, tmin=tmin, tmax=tmax, seed=seed)
        self.img, self.num_ray, self.mix, self.amp = img, num_ray, mix, amplitude
        self.rng = np.random.default_rng(seed + 1)
        self.cams = [np.ascontiguousarray(workloads.box_ortho_ndc2world(v.min(0), v.max(0))) for _, v in self.meshes]
        self.max_tri = max(t.shape[0] for t, _ in self.meshes)
        self.max_out = max(img * img, num_ray)
        self.rays = {}
        self._outs = [pinned((self.max_out,), np.uint32) for _ in range(ring)]
        self._frames = np.zeros(num_mesh, np.int64)

    def register_all(self, server: Server):
        for i, (t, v) in enumerate(self.meshes):
            server.register(i, t, v, seed=1000 + i)

    def _ray_set(self, m):
        if m not in self.rays:
            lo, hi = self.meshes[m][1].min(0), self.meshes[m][1].max(0)
            org, d = workloads.cube_boundary_rays(self.num_ray, seed=m)
            org = (lo + org * (hi - lo)).astype(np.float32)
            ot, oa = pinned(org.shape, np.float32)
            dt_, da = pinned(d.shape, np.float32)
            oa[:] = org
            da[:] = d
            self.rays[m] = (ot, oa, dt_, da)
        return self.rays[m]

    def request(self, kind, m, frame, out=None):
        r = Request()
        r.kind, r.mesh_id, r.frame, r.deform_amplitude = kind, m, frame, self.amp
        if kind == CAST_RAYS:
            _, oa, _, da = self._ray_set(m)
            r.num_ray, r.ray_org, r.ray_dir = self.num_ray, oa.ctypes.data, da.ctypes.data
        else:
            r.img_w = r.img_h = self.img
            r.transform_ndc2world = self.cams[m].ctypes.data
        if out is None:
            out = self._outs[self.rng.integers(len(self._outs))][1]
        r.out_tri = out.ctypes.data
        r.out_t = None
        return r

    def stream(self, n, rate_hz, zipf: float = 0.0):
        """n requests with Poisson arrivals at rate_hz; mesh ids uniform over the
        pool; each refit advances that mesh's frame."""
        arr = np.cumsum(self.rng.exponential(1.0 / rate_hz, n))
        kinds = self.rng.choice(3, size=n, p=self.mix)
        mids = self.rng.integers(0, len(self.meshes), n)
        reqs = []
        for k, m in zip(kinds, mids):
            if k == REFIT_CAST:
                self._frames[m] += 1
            reqs.append(self.request(int(k), int(m), int(self._frames[m])))
        return reqs, arr
