#!/usr/bin/env python
"""Benchmark of the LBVH build + BVH ray cast on one GB300 (or N replicas).

Workload (one "step"): the 2,097,152-triangle displaced torus (1024x1024 quad
grid, R=1, r=0.3, seeded radial displacement of amplitude 0.02 with 8 integer
frequencies in 1..64) gets a full LBVH build (centroids, fit, Morton codes,
radix sort, topology, AABBs) and a 1920x1080 pinhole cast (60 degree vertical
FOV from a seeded viewpoint on the radius-3 sphere), writing the hit triangle
id and hit t of every pixel.  Inputs are seeded synthetic meshes of that shape.

Metric: rays/s of the whole step (build included), the aggregate over all
ranks.  Also reported: build-only triangles/s, cast-only rays/s, per-stage
times, the HBM roofline of the dominant kernel, an end-to-end figure through
the public torch API with host buffers, and the oracle (CPU restatement of
del-msh-cpu) timed on the host cores.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With --impl reference the CPU restatement of del-msh-cpu's path (the oracle)
runs the same workload on the host cores (build on one thread as in the
reference, cast on every host thread as rayon does) and prints the same line.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import pathlib
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = pathlib.Path(__file__).resolve().parent
for _p in (ROOT, ROOT / "del-msh_gb300"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

import numpy as np  # noqa: E402

METRIC = "rays/s (LBVH build + cast per step)"
UNIT = "rays/s"
IMG_W, IMG_H = 1920, 1080
# kernels of this repo launched per single-mesh step: build = centroid AABB,
# Morton, 4 sort passes, topology, 6 refit kernels (window, superblock, the
# two crossing-branch kernels, and the tree-order climb's two, which exit at
# once without NaN); cast = persistent traversal + the warp tier + 2 serial
# overflow tiers (the last three exit at once when their lists are empty)
KERNELS_PER_STEP = 17
NDIV = 1024
SEED = 0
L2_FLUSH_BYTES = 256 << 20


def workload():
    from del_msh_gb300 import workloads as W
    tri, vtx = W.displaced_torus(NDIV, seed=SEED)
    m = W.pinhole_ndc2world(W.random_viewpoint(3.0, seed=SEED), aspect=IMG_W / IMG_H)
    return tri, vtx, m


def config_dict(tri, vtx):
    return {
        "workload": "displaced torus 1024x1024 grid (2,097,152 tris) LBVH build + 1920x1080 pinhole cast",
        "num_tri": int(tri.shape[0]), "num_vtx": int(vtx.shape[0]), "rays_per_step": IMG_W * IMG_H,
        "seed": SEED, "l2": "flushed between timed steps (256 MiB write)",
    }


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def algorithmic_bytes(T: int, V: int, R: int):
    """Compulsory DRAM bytes per launch of each stage (u32/f32 = 4 B)."""
    return {
        # centroid AABB pass (stores the centroids) + Morton pass (reads them; codes and histograms)
        "morton": (12 * T + 12 * V + 12 * T) + (12 * T + 8 * T),
        "sort": 68 * T,  # 4T histogram + 4 passes x (8T read + 8T write)
        "topology": 8 * T + 24 * T,
        "refit": 24 * T + 12 * T + 12 * V + 48 * T + 8 * T,
        "build": 236 * T + 24 * V,
        "cast": 8 * R + 72 * T + 12 * T + 12 * V,  # outputs + one read of tree and mesh
    }


# --------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100", "-f", self.path], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in pathlib.Path(self.path).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# -------------------------------------------------------------- CPU side

def cpu_step(O, tri, vtx, m, threads: int, keep=None):
    """One oracle step: build on one thread (as del-msh-cpu), cast on `threads`."""
    t0 = time.perf_counter()
    r = O.build(tri, vtx)
    t1 = time.perf_counter()
    out = O.pix2tri(tri, vtx, r["bvhnodes"], r["bvhnode2aabb"], m, IMG_W, IMG_H, threads=threads)
    t2 = time.perf_counter()
    if keep is not None:
        keep[:] = [np.asarray(out[0]).reshape(-1).view(np.uint32), np.asarray(out[1]).reshape(-1)]
    return t1 - t0, t2 - t1


def cpu_baseline(tri, vtx, m, reps: int = 3):
    from oracle import build as obuild
    from oracle import oracle as O
    obuild.build_oracle()
    threads = O.default_threads()
    cpu_step(O, tri, vtx, m, threads)  # warm-up
    builds, casts = [], []
    keep = []
    for _ in range(reps):
        b, c = cpu_step(O, tri, vtx, m, threads, keep=keep)
        builds.append(b)
        casts.append(c)
    b, c = statistics.median(builds), statistics.median(casts)
    return ({"value": IMG_W * IMG_H / (b + c), "unit": UNIT, "cores": threads, "kind": "port",
             "sample": f"the full step (build on 1 thread, 1920x1080 cast on {threads} threads), median of {reps}",
             "build_tris_per_s": tri.shape[0] / b, "cast_rays_per_s": IMG_W * IMG_H / c}, tuple(keep))


# ------------------------------------------------------------- GPU side

def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def reduce_max_over_ranks(pg, values, device=None):
    """Each value's maximum over the ranks: the slowest replica sets the job's
    time.  pg is torch.distributed (or None for one process)."""
    if pg is None:
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def job_throughput(world: int, units_per_rank: float, ms: float) -> float:
    """Whole-job units/s of `world` replicas that each process units_per_rank
    in ms (the max over ranks)."""
    return world * units_per_rank / (ms * 1e-3)


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import build as obuild
    from oracle import oracle as O
    obuild.build_oracle()
    tri, vtx, m = workload()
    threads = O.default_threads()
    for _ in range(args.warmup):
        cpu_step(O, tri, vtx, m, threads)
    t0 = time.perf_counter()
    builds, casts = [], []
    for _ in range(args.steps):
        b, c = cpu_step(O, tri, vtx, m, threads)
        builds.append(b)
        casts.append(c)
    total = time.perf_counter() - t0
    step_s = total / args.steps
    value = IMG_W * IMG_H / step_s
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32/u32", "data": "synthetic (seeded displaced torus)",
        "config": config_dict(tri, vtx), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full steps (build on 1 thread as del-msh-cpu, cast on {threads} "
                                   f"threads as its rayon loop)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "build_tris_per_s": tri.shape[0] / statistics.mean(builds),
        "cast_rays_per_s": IMG_W * IMG_H / statistics.mean(casts),
        "note": "del-msh-cpu (Rust) cannot be built here; the oracle is its C restatement, bit-exact on this path",
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
        pg = dist
    from del_msh_gb300 import _native
    from del_msh_gb300.Pix2Tri import torch as Pix2Tri
    from del_msh_gb300.TriMesh3 import torch as TriMesh3

    L = _native.load(build_if_missing=True)
    tri, vtx, m = workload()
    T, V, R = tri.shape[0], vtx.shape[0], IMG_W * IMG_H
    d_tri = torch.from_numpy(tri.view(np.int32)).to(dev).view(torch.uint32)
    d_vtx = torch.from_numpy(vtx).to(dev)
    d_m = torch.from_numpy(m).to(dev)  # column-major, as the C ABI reads it
    bvh = torch.empty((2 * T - 1, 3), dtype=torch.int32, device=dev)
    aabb = torch.empty((2 * T - 1, 6), dtype=torch.float32, device=dev)
    pix2tri = torch.empty((IMG_H, IMG_W), dtype=torch.int32, device=dev)
    pix2t = torch.empty((IMG_H, IMG_W), dtype=torch.float32, device=dev)
    bs = L.dm_trimesh3_build_scratch_bytes(T)
    cs = L.dm_cast_scratch_bytes(R, T)
    b_scratch = torch.empty((bs,), dtype=torch.uint8, device=dev)
    c_scratch = torch.empty((cs,), dtype=torch.uint8, device=dev)
    flush = torch.empty((L2_FLUSH_BYTES,), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream

    def build():
        _native.call("dm_trimesh3_make_bvhnodes_bvhnode2aabb", sp, T, d_tri.data_ptr(), V, d_vtx.data_ptr(),
                     bvh.data_ptr(), aabb.data_ptr(), b_scratch.data_ptr(), bs)

    def cast():
        _native.call("dm_pix2tri_by_raycast", sp, IMG_W, IMG_H, pix2tri.data_ptr(), pix2t.data_ptr(), T,
                     d_tri.data_ptr(), V, d_vtx.data_ptr(), bvh.data_ptr(), aabb.data_ptr(), d_m.data_ptr(),
                     c_scratch.data_ptr(), cs)

    for _ in range(max(args.warmup, 3)):
        flush.zero_()
        build()
        cast()
    torch.cuda.synchronize()

    def barrier():
        if pg is not None:
            pg.barrier()
        torch.cuda.synchronize()

    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    sampler = ClockSampler(local)
    sampler.start()
    barrier()
    wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()  # L2 flush, outside the event pair
        ev[k][0].record(stream)
        build()
        ev[k][1].record(stream)
        cast()
        ev[k][2].record(stream)
    barrier()
    wall = time.perf_counter() - wall0
    clocks = sampler.stop()
    build_ms = [ev[k][0].elapsed_time(ev[k][1]) for k in range(args.steps)]
    cast_ms = [ev[k][1].elapsed_time(ev[k][2]) for k in range(args.steps)]
    step_ms = statistics.mean(b + c for b, c in zip(build_ms, cast_ms))
    build_mean, cast_mean = statistics.mean(build_ms), statistics.mean(cast_ms)

    # correctness guard on the timed outputs: status word clean
    status = _native.device_status(clear=True)

    # per-stage breakdown of the build (CUDA events between stages)
    stage = (ctypes.c_float * 4)()
    stage_runs = []
    for _ in range(max(3, min(args.steps, 20))):
        flush.zero_()
        _native.call("dm_trimesh3_build_profiled", sp, T, d_tri.data_ptr(), V, d_vtx.data_ptr(), bvh.data_ptr(),
                     aabb.data_ptr(), b_scratch.data_ptr(), bs, ctypes.cast(stage, ctypes.c_void_p))
        stage_runs.append(list(stage))
    stage_ms = {k: statistics.mean(r[i] for r in stage_runs)
                for i, k in enumerate(("morton", "sort", "topology", "refit"))}

    # refit-only deformed frame through the drop-in refit (the reference's
    # bvhnode2aabb_update_aabb): v += 0.01 sin(phase + frame), resident tree
    phase = np.random.default_rng(SEED + 7).uniform(0.0, 2.0 * np.pi, V)
    d_def = torch.from_numpy((vtx + 0.01 * np.sin(phase + 1.0)[:, None]).astype(np.float32)).to(dev)
    rs = L.dm_bvhnode2aabb_update_aabb_scratch_bytes(T)
    r_scratch = torch.zeros((rs,), dtype=torch.uint8, device=dev)
    r_aabb = torch.empty_like(aabb)

    def refit_frame():
        _native.call("dm_bvhnode2aabb_update_aabb_ex", sp, 2 * T - 1, r_aabb.data_ptr(), bvh.data_ptr(), T,
                     d_tri.data_ptr(), V, d_def.data_ptr(), None, r_scratch.data_ptr(), rs)

    for _ in range(3):
        refit_frame()
    r_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for a, z in r_ev:
        flush.zero_()
        a.record(stream)
        refit_frame()
        z.record(stream)
    torch.cuda.synchronize()
    refit_frame_ms = statistics.mean(a.elapsed_time(z) for a, z in r_ev)
    del r_scratch, r_aabb, d_def

    # end to end through the public torch API with host buffers
    h_tri = torch.from_numpy(tri.view(np.int32)).pin_memory()
    h_vtx = torch.from_numpy(vtx).pin_memory()
    m_row = torch.from_numpy(np.ascontiguousarray(m.reshape(4, 4).T)).to(dev)
    e_tri = torch.empty_like(d_tri.view(torch.int32))
    e_vtx = torch.empty_like(d_vtx)
    h_p2t = torch.empty((IMG_H, IMG_W), dtype=torch.int32).pin_memory()
    h_tt = torch.empty((IMG_H, IMG_W), dtype=torch.float32).pin_memory()

    def e2e_step():
        e_tri.copy_(h_tri, non_blocking=True)
        e_vtx.copy_(h_vtx, non_blocking=True)
        t_tri = e_tri.view(torch.uint32)
        b2, a2 = TriMesh3.make_bvhnodes_bvhnode2aabb(t_tri, e_vtx)
        p2, t2 = Pix2Tri.by_raycasting(t_tri, e_vtx, b2, a2, m_row, (IMG_W, IMG_H), return_depth=True)
        h_p2t.copy_(p2.view(torch.int32), non_blocking=True)
        h_tt.copy_(t2, non_blocking=True)

    for _ in range(3):
        e2e_step()
    barrier()
    e_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for k in range(args.steps):
        flush.zero_()
        e_ev[k][0].record(stream)
        e2e_step()
        e_ev[k][1].record(stream)
    barrier()
    e2e_serial_ms = statistics.mean(a.elapsed_time(b) for a, b in e_ev)
    ok = bool(np.array_equal(h_p2t.numpy(), pix2tri.cpu().numpy()))

    # The same calls as a serving loop runs them back to back: step k+1's
    # upload (copy stream) overlaps step k's build + cast (compute stream),
    # and step k's download (a second copy stream) overlaps step k+1.  Device
    # inputs and pinned outputs are double-buffered; every step still copies
    # its whole mesh in and its whole image out inside the timed region.
    s_in, s_out = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    p_tri = [e_tri, torch.empty_like(e_tri)]
    p_vtx = [e_vtx, torch.empty_like(e_vtx)]
    p_hp = [h_p2t, torch.empty_like(h_p2t).pin_memory()]
    p_ht = [h_tt, torch.empty_like(h_tt).pin_memory()]
    consumed = [torch.cuda.Event(), torch.cuda.Event()]  # compute finished with input buffer b

    def pipelined(steps):
        ev_start, ev_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev_start.record(stream)
        s_in.wait_event(ev_start)
        for k in range(steps):
            b = k & 1
            with torch.cuda.stream(s_in):
                if k >= 2:
                    s_in.wait_event(consumed[b])
                p_tri[b].copy_(h_tri, non_blocking=True)
                p_vtx[b].copy_(h_vtx, non_blocking=True)
                uploaded = torch.cuda.Event()
                uploaded.record(s_in)
            stream.wait_event(uploaded)
            t_tri = p_tri[b].view(torch.uint32)
            b2, a2 = TriMesh3.make_bvhnodes_bvhnode2aabb(t_tri, p_vtx[b])
            p2, t2 = Pix2Tri.by_raycasting(t_tri, p_vtx[b], b2, a2, m_row, (IMG_W, IMG_H), return_depth=True)
            consumed[b].record(stream)
            computed = torch.cuda.Event()
            computed.record(stream)
            with torch.cuda.stream(s_out):
                s_out.wait_event(computed)
                p_hp[b].copy_(p2.view(torch.int32), non_blocking=True)
                p_ht[b].copy_(t2, non_blocking=True)
                p2.record_stream(s_out)
                t2.record_stream(s_out)
        ev_end.record(s_out)
        ev_end.synchronize()
        return ev_start.elapsed_time(ev_end) / steps

    pipelined(3)
    barrier()
    e2e_ms = pipelined(args.steps)
    barrier()
    ok = ok and bool(np.array_equal(p_hp[(args.steps - 1) & 1].numpy(), pix2tri.cpu().numpy()))

    step_ms, e2e_ms, e2e_serial_ms, build_mean, cast_mean = reduce_max_over_ranks(
        pg, [step_ms, e2e_ms, e2e_serial_ms, build_mean, cast_mean], dev)
    if rank != 0:
        if pg is not None:
            pg.destroy_process_group()
        return 0

    nbytes = algorithmic_bytes(T, V, R)
    peak, peak_kind = peaks()
    stage_all = dict(stage_ms, cast=cast_mean)
    dom = max(stage_all, key=stage_all.get)
    dom_ms = stage_all[dom]
    traffic = read_traffic(dom)
    achieved = nbytes[dom] / (dom_ms * 1e-3) / 1e9
    build_gbs = nbytes["build"] / (build_mean * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": job_throughput(world, R, step_ms), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32/u32", "data": "synthetic (seeded displaced torus)",
        "config": config_dict(tri, vtx),
        "build_tris_per_s": world * T / (build_mean * 1e-3), "cast_rays_per_s": world * R / (cast_mean * 1e-3),
        "build_ms": build_mean, "cast_ms": cast_mean, "stage_ms": stage_ms,
        "refit_frame": {"ms": refit_frame_ms, "tris_per_s": T / (refit_frame_ms * 1e-3),
                        "api": "dm_bvhnode2aabb_update_aabb_ex (drop-in refit: leaf ranges derived from bvhnodes, "
                               "then range queries)",
                        "workload": "deformed frame v += 0.01 sin(phase + 1) of the torus, resident tree, "
                                    "L2 flushed"},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": f"{peak_kind} hbm_gbs",
                     "algorithmic_bytes": nbytes[dom]},
        "build_roofline": {"achieved": build_gbs, "peak": peak, "unit": "GB/s", "frac": build_gbs / peak,
                           "algorithmic_bytes": nbytes["build"]},
        "e2e": {"value": job_throughput(world, R, e2e_ms), "unit": UNIT,
                "h2d_bytes_per_step": int(tri.nbytes + vtx.nbytes), "d2h_bytes_per_step": int(8 * R),
                "ms_per_step": e2e_ms, "api": "TriMesh3.torch + Pix2Tri.torch", "matches_device_run": ok,
                "schedule": "pipelined: step k+1's upload and step k's download (two copy streams) overlap the "
                            "build + cast (compute stream); inputs and outputs double-buffered; no L2 flush "
                            "between steps (each step touches ~220 MB, more than the 129 MB L2)",
                "serial": {"value": job_throughput(world, R, e2e_serial_ms), "ms_per_step": e2e_serial_ms,
                           "schedule": "upload, build, cast, download on one stream; L2 flushed between steps"}},
        "gpu_launches": args.steps * KERNELS_PER_STEP,
        "tuning": _native.get_tuning(),
        "clocks": clocks,
        "device_status": status,
        "wall_s": wall,
    }
    g_p2t = pix2tri.cpu().numpy().view(np.uint32).reshape(-1)
    g_tt = pix2t.cpu().numpy().reshape(-1)
    line["t_error_f64"] = {"gpu": t_error_f64(np.asarray(m), IMG_W, IMG_H, g_p2t, g_tt, tri, vtx),
                           "definition": "relative error of the f32 hit t against the same pixel ray and "
                                         "Moller-Trumbore formula evaluated in binary64, over every hit pixel"}
    if not args.no_cpu:
        line["cpu_baseline"], (c_p2t, c_tt) = cpu_baseline(tri, vtx, np.asarray(m))
        line["t_error_f64"]["cpu"] = t_error_f64(np.asarray(m), IMG_W, IMG_H, c_p2t, c_tt, tri, vtx)
        line["t_error_f64"]["cpu_bits_equal_gpu"] = bool(np.array_equal(c_p2t, g_p2t) and
                                                         np.array_equal(c_tt.view(np.uint32), g_tt.view(np.uint32)))
    if not args.no_extras and world == 1:
        del b_scratch, c_scratch, bvh, aabb, d_tri, d_vtx
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        line.update(compact_extras(args))
    print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()
    return 0


def t_error_f64(m, img_w, img_h, p2t, tt, tri, vtx):
    """Max / median / p99 relative error of the f32 hit t of every hit pixel
    against binary64: the pixel ray (ray_for_pixel's formula) and the
    Moller-Trumbore t of the hit triangle, both evaluated in float64."""
    idx = np.flatnonzero(p2t != 0xFFFFFFFF)
    if idx.size == 0:
        return {"hits": 0}
    ih = idx // img_w
    iw = idx - ih * img_w
    x0 = 2.0 * (iw + 0.5) / img_w - 1.0
    y0 = 1.0 - 2.0 * (ih + 0.5) / img_h
    mm = np.asarray(m, np.float64).reshape(4, 4).T  # column-major storage -> row-major matrix
    one = np.ones_like(x0)
    q0 = np.stack([x0, y0, one, one], 1) @ mm.T
    q1 = np.stack([x0, y0, -one, one], 1) @ mm.T
    org = q0[:, :3] / q0[:, 3:4]
    d = q1[:, :3] / q1[:, 3:4] - org
    t3 = tri[p2t[idx]].astype(np.int64)
    v = vtx.astype(np.float64)
    p0, p1, p2 = v[t3[:, 0]], v[t3[:, 1]], v[t3[:, 2]]
    e1, e2 = p1 - p0, p2 - p0
    pv = np.cross(d, e2)
    det = (e1 * pv).sum(1)
    qv = np.cross(org - p0, e1)
    t64 = (e2 * qv).sum(1) / det
    rel = np.abs(tt[idx].astype(np.float64) - t64) / np.abs(t64)
    return {"hits": int(idx.size), "max_rel": float(rel.max()), "median_rel": float(np.median(rel)),
            "p99_rel": float(np.percentile(rel, 99))}


def compact_extras(args):
    """The other workloads, measured after the headline step in the
    same process and reported as compact keys of the same line: the ragged
    batch (graph replay against the plain per-mesh path), the served stream
    (p50/p99 at 0.5x and 0.8x of the plain path's capacity) and the
    adversarial soup (build and cast times).  A failure is reported in the key
    instead of aborting the line."""
    out = {}
    try:
        bt = measure_batched(4096, steps=10, warmup=2, plain_steps=2)
        out["batched"] = {"num_mesh": bt["config"]["num_mesh"], "total_tri": bt["config"]["total_tri"],
                          "rays_per_step": bt["config"]["rays_per_step"],
                          "graph_ms_per_step": bt["batched_graph"]["ms_per_step"],
                          "graph_rays_per_s": bt["batched_graph"]["rays_per_s"],
                          "graph_tris_per_s": bt["batched_graph"]["tris_per_s"],
                          "plain_ms_per_step": max(bt["plain"]["ms_per_step_device"], bt["plain"]["ms_per_step_wall"]),
                          "plain_rays_per_s": bt["plain"]["rays_per_s"],
                          "speedup_vs_plain": bt["speedup_vs_plain"],
                          "outputs_identical_to_plain": bt["outputs_identical_to_plain"],
                          "device_status": bt["device_status"]}
    except Exception as e:  # noqa: BLE001 - reported, not raised
        out["batched"] = {"error": f"{type(e).__name__}: {e}"}
    try:
        sv = measure_served(512, 600, [0.5, 0.8], 8, 120.0)
        loads = []
        for ld in sv["loads"]:
            e = {"fraction_of_plain_capacity": ld["fraction_of_plain_capacity"], "offered_rps": ld["offered_rps"],
                 "served_p50_ms": ld["served"]["p50_ms"], "served_p99_ms": ld["served"]["p99_ms"],
                 "served_rays_per_s": ld["served_rays_per_s"]}
            if "plain" in ld:
                e.update({"plain_p50_ms": ld["plain"]["p50_ms"], "plain_p99_ms": ld["plain"]["p99_ms"],
                          "plain_rays_per_s": ld["plain_rays_per_s"],
                          "served_p99_below_plain_p50": ld["served_p99_below_plain_p50"]})
            loads.append(e)
        out["served"] = {"pool": sv["config"]["pool"], "total_tri": sv["config"]["total_tri"],
                         "plain_capacity_rps": sv["plain_capacity_rps"],
                         "served_capacity_rps": sv["served_capacity_rps"], "loads": loads,
                         "requests_per_trace": sv["config"]["requests_per_trace"],
                         "device_status": sv["device_status"]}
    except Exception as e:  # noqa: BLE001
        out["served"] = {"error": f"{type(e).__name__}: {e}"}
    try:
        sp = measure_soup(steps=5, warmup=3, cpu=False)
        out["soup"] = {"num_tri": sp["config"]["num_tri"], "rays": sp["config"]["rays"], "build_ms": sp["build_ms"],
                       "cast_ms": sp["cast_ms"], "rays_per_s": sp["value"],
                       "build_roofline_frac": sp["build_roofline_frac"], "device_status": sp["device_status"]}
    except Exception as e:  # noqa: BLE001
        out["soup"] = {"error": f"{type(e).__name__}: {e}"}
    return out


def run_batched(args):
    print(json.dumps(measure_batched(args.num_mesh, args.steps, args.warmup)), flush=True)
    return 0


def measure_batched(num_mesh: int, steps: int, warmup: int, plain_steps: int | None = None):
    """Ragged batch: ``num_mesh`` seeded jittered icospheres / tori, triangle
    counts log-uniform in [64, 65536] (37.9M triangles for 4096 meshes), each
    with its own 64x64 orthographic image.  One step = build every tree + cast
    every image.  Timed three ways on the same GPU: the plain path (one launch
    sequence per mesh through the single-mesh entry points), the batched entry
    points called eagerly, and the batched step replayed from a CUDA graph."""
    import torch
    from del_msh_gb300 import _native
    from del_msh_gb300 import workloads as W
    from del_msh_gb300.batch import MeshBatch, PlainPath, ortho_transforms
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    _native.load(build_if_missing=True)
    t0 = time.perf_counter()
    meshes = W.ragged_batch(num_mesh=num_mesh, tmin=64, tmax=65536, seed=SEED)
    gen_s = time.perf_counter() - t0
    b = MeshBatch(meshes, dev)
    tf = torch.from_numpy(ortho_transforms(meshes)).to(dev)
    b.alloc_cast(64, 64)
    plain = PlainPath(b)
    plain.alloc_cast(64, 64)
    R = b.num_mesh * 64 * 64
    stream = torch.cuda.current_stream(dev)

    def timed(fn, steps):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        for a, z in evs:
            a.record(stream)
            fn()
            z.record(stream)
        torch.cuda.synchronize()
        wall = (time.perf_counter() - w0) / steps
        return statistics.mean(a.elapsed_time(z) for a, z in evs), wall * 1e3

    def plain_step():
        plain.build()
        plain.cast_pixels(tf)

    def batch_step():
        # an NVTX range, so that a profiler can keep this step's launches
        # apart from the plain path's (ncu --nvtx --nvtx-include "batched step/")
        torch.cuda.nvtx.range_push("batched step")
        b.build()
        b.cast_pixels(tf)
        torch.cuda.nvtx.range_pop()

    for _ in range(max(1, warmup // 2)):
        plain_step()
        batch_step()
    b.capture(tf)
    b.replay()
    torch.cuda.synchronize()
    plain_ms, plain_wall = timed(plain_step, plain_steps or max(2, steps // 10))
    eager_ms, eager_wall = timed(batch_step, steps)
    graph_ms, graph_wall = timed(b.replay, steps)
    match = bool(torch.equal(b.pix2tri.view(torch.int32), plain.pix2tri.view(torch.int32)) and
                 torch.equal(b.pix2t, plain.pix2t))
    status = _native.device_status(clear=True)
    plain_eff = max(plain_ms, plain_wall)
    line = {
        "metric": "rays/s (batched LBVH build + cast of ragged meshes)", "unit": UNIT,
        "value": R / (graph_ms * 1e-3), "n_gpus": 1, "steps": steps, "warmup": warmup,
        "ms_per_step": graph_ms, "higher_is_better": True, "dtype": "f32/u32",
        "data": "synthetic (seeded jittered icospheres / tori)",
        "config": {"workload": f"{b.num_mesh} ragged meshes, triangle counts log-uniform in [64, 65536], "
                               f"64x64 orthographic rays each", "num_mesh": b.num_mesh,
                   "total_tri": b.total_tri, "rays_per_step": R, "generation_s": gen_s},
        "plain": {"ms_per_step_device": plain_ms, "ms_per_step_wall": plain_wall,
                  "rays_per_s": R / (plain_eff * 1e-3), "tris_per_s": b.total_tri / (plain_eff * 1e-3)},
        "batched_eager": {"ms_per_step": eager_ms, "ms_per_step_wall": eager_wall,
                          "rays_per_s": R / (max(eager_ms, eager_wall) * 1e-3)},
        "batched_graph": {"ms_per_step": graph_ms, "ms_per_step_wall": graph_wall,
                          "rays_per_s": R / (max(graph_ms, graph_wall) * 1e-3),
                          "tris_per_s": b.total_tri / (graph_ms * 1e-3)},
        "speedup_vs_plain": plain_eff / max(graph_ms, graph_wall),
        "outputs_identical_to_plain": match, "device_status": status,
    }
    del b, plain
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return line


def run_served(args):
    print(json.dumps(measure_served(args.pool, args.requests, args.loads, args.slots, args.budget_gb)), flush=True)
    return 0


def measure_served(pool: int, requests: int, loads, slots: int, budget_gb: float):
    """Served configuration: a pool of 512 seeded icospheres / tori (triangle
    counts log-uniform in [1k, 1M]), Poisson arrivals, 20% build + 512x512
    cast, 60% refit + re-cast after a per-frame deformation of the resident
    tree, 20% cast of 16k random rays; 120 GB HBM budget with LRU eviction.
    The request server and the plain serial path run the same traces at the
    same offered loads on the same GPU; latency counts from the scheduled
    arrival to the completion of the result download."""
    import torch
    from del_msh_gb300 import _native
    from del_msh_gb300.serve import Server, ServedWorkload, latency_stats
    torch.cuda.set_device(0)
    _native.load(build_if_missing=True)
    t0 = time.perf_counter()
    wl = ServedWorkload(num_mesh=pool, tmin=1000, tmax=1_000_000, img=512, num_ray=16384, seed=SEED)
    gen_s = time.perf_counter() - t0
    n = requests
    out = {"metric": "served requests: p50/p99 latency and rays/s against the plain serial path", "unit": "ms",
           "config": {"pool": pool, "total_tri": int(sum(t.shape[0] for t, _ in wl.meshes)),
                      "max_tri": wl.max_tri, "mix": "20% build+cast 512^2, 60% refit+re-cast, 20% cast 16k rays",
                      "budget_gb": budget_gb, "slots": slots, "requests_per_trace": n,
                      "generation_s": gen_s}, "data": "synthetic (seeded jittered icospheres / tori)",
           "loads": []}
    with Server(budget_bytes=int(budget_gb * (1 << 30)), num_slots=slots, max_tri=wl.max_tri,
                max_out=wl.max_out) as srv:
        wl.register_all(srv)
        # capacities: a closed burst (all arrivals at t=0) through each path
        reqs, _ = wl.stream(min(n, 300), 1.0)
        plain_burst = latency_stats(srv.run_plain(reqs, [0.0] * len(reqs)))
        plain_cap = len(reqs) / plain_burst["span_s"]
        # build every mesh of the pool once, so that the traces run on
        # resident trees (the configuration's refit and cast requests name a
        # resident BVH) and no admission falls inside a timed trace
        reqs = [wl.request(0, m, 0) for m in range(len(wl.meshes))]
        srv.run_trace(reqs, [0.0] * len(reqs))
        reqs, _ = wl.stream(n, 1.0)
        served_burst = latency_stats(srv.run_trace(reqs, [0.0] * n))
        served_cap = n / served_burst["span_s"]
        out["plain_capacity_rps"] = plain_cap
        out["served_capacity_rps"] = served_cap
        for frac in loads:
            rate = frac * plain_cap
            reqs, arr = wl.stream(n, rate)
            rays = sum(r.num_ray if r.kind == 2 else r.img_w * r.img_h for r in reqs)
            s = latency_stats(srv.run_trace(reqs, arr), kinds=[r.kind for r in reqs])
            entry = {"offered_rps": rate, "fraction_of_plain_capacity": frac, "served": s,
                     "served_rays_per_s": rays / s["span_s"]}
            if frac <= 0.9:
                reqs_p, arr_p = wl.stream(min(n, 600), rate)
                rays_p = sum(r.num_ray if r.kind == 2 else r.img_w * r.img_h for r in reqs_p)
                p = latency_stats(srv.run_plain(reqs_p, arr_p), kinds=[r.kind for r in reqs_p])
                entry["plain"] = p
                entry["plain_rays_per_s"] = rays_p / p["span_s"]
                entry["served_p99_below_plain_p50"] = s["p99_ms"] < p["p50_ms"]
            out["loads"].append(entry)
        out["server_stats"] = srv.stats()
    from del_msh_gb300 import _native as N
    out["device_status"] = N.device_status(clear=True)
    del wl
    import torch
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return out


def run_render(args):
    """The consumers of the torus's pix2tri image (1920x1080 over the
    2,097,152-triangle torus): depth and 3-channel interpolation, forward and
    backward, each timed alone with CUDA events (L2 flushed between
    repetitions), with the oracle on the host cores beside them."""
    import torch
    from del_msh_gb300 import _native
    from del_msh_gb300.Pix2Depth import torch as Pix2Depth
    from del_msh_gb300.Pix2Tri import torch as Pix2Tri
    from del_msh_gb300.TriMesh3 import torch as TriMesh3
    dev = torch.device("cuda", 0)
    _native.load(build_if_missing=True)
    tri, vtx, m = workload()
    T, V, R = tri.shape[0], vtx.shape[0], IMG_W * IMG_H
    d_tri = torch.from_numpy(tri.view(np.int32)).to(dev).view(torch.uint32)
    d_vtx = torch.from_numpy(vtx).to(dev)
    m_row = torch.from_numpy(np.ascontiguousarray(np.asarray(m).reshape(4, 4).T)).to(dev)
    bvh, aabb = TriMesh3.make_bvhnodes_bvhnode2aabb(d_tri, d_vtx)
    p2t = Pix2Tri.by_raycasting(d_tri, d_vtx, bvh, aabb, m_row, (IMG_W, IMG_H))
    nd = 3
    val = torch.rand((V, nd), device=dev)
    depth = torch.zeros((IMG_H, IMG_W), device=dev)
    g_depth = torch.rand((IMG_H, IMG_W), device=dev)
    g_val = torch.rand((IMG_H, IMG_W, nd), device=dev)
    gx = torch.zeros((V, 3), device=dev)
    gv = torch.zeros((V, nd), device=dev)
    flush = torch.empty((L2_FLUSH_BYTES,), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    ops = {
        "depth_fwd": lambda: Pix2Depth.update(depth, p2t, d_tri, d_vtx, m_row),
        "depth_bwd": lambda: Pix2Depth.bwd_wrt_vtx2xyz(gx, p2t, d_tri, d_vtx, g_depth, m_row),
        "interp_fwd": lambda: Pix2Tri.interpolate_fwd(p2t, d_tri, d_vtx, val, m_row),
        "interp_bwd": lambda: Pix2Tri.interpolate_bwd(p2t, d_tri, d_vtx, val, m_row, g_val, gx, gv),
    }
    hits = int((p2t != torch.iinfo(torch.uint32).max).sum().item())
    # compulsory bytes per pixel: pix2tri 4 + (hit pixels) triangle 12 + 3 vertices 36 (+ values / grads)
    per_hit = {"depth_fwd": 48, "depth_bwd": 48 + 36, "interp_fwd": 48 + 12 * nd,
               "interp_bwd": 48 + 12 * nd + 36 + 12 * nd}
    per_pix = {"depth_fwd": 4 + 4, "depth_bwd": 4 + 4, "interp_fwd": 4 + 4 * nd, "interp_bwd": 4 + 4 * nd}
    peak, peak_kind = peaks()
    res = {}
    for name, fn in ops.items():
        for _ in range(max(args.warmup, 3)):
            fn()
        times = []
        for _ in range(args.steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
        ms = statistics.median(times)
        nbytes = per_pix[name] * R + per_hit[name] * hits
        res[name] = {"ms": ms, "pixels_per_s": R / (ms * 1e-3), "algorithmic_bytes": nbytes,
                     "hbm_frac": nbytes / (ms * 1e-3) / 1e9 / peak}
    status = _native.device_status(clear=True)
    line = {"metric": "pixels/s (depth / interpolation from a 1920x1080 pix2tri image, fwd and bwd)",
            "unit": "pixels/s", "value": res["interp_fwd"]["pixels_per_s"], "steps": args.steps,
            "config": {"workload": "displaced torus (2,097,152 tris), 1920x1080 pinhole pix2tri, 3 value channels",
                       "hit_pixels": hits, "l2": "flushed between repetitions"},
            "ops": res, "peak": {"hbm_gbs": peak, "kind": peak_kind}, "device_status": status,
            "note": "backward passes accumulate with atomicAdd, as the reference's kernels do"}
    if not args.no_cpu:
        from oracle import build as obuild
        from oracle import oracle as O
        obuild.build_oracle()
        h_p2t = p2t.cpu().numpy()
        hv, hg = val.cpu().numpy(), g_val.cpu().numpy()
        t0 = time.perf_counter()
        O.interpolate(h_p2t, tri, vtx, hv, np.asarray(m), IMG_W, IMG_H)
        t_f = time.perf_counter() - t0
        t0 = time.perf_counter()
        O.interpolate_bwd(h_p2t, tri, vtx, hv, np.asarray(m), hg, IMG_W, IMG_H)
        t_b = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": R / t_f, "unit": "pixels/s", "cores": 1, "kind": "port",
                                "sample": "one interpolation forward of the full image (1 thread)",
                                "interp_bwd_pixels_per_s": R / t_b}
    print(json.dumps(line), flush=True)
    return 0


def run_octree(args):
    """Quad/oct-tree construction from 2,097,152 sorted unique 30-bit Morton
    codes (3-D, uniform random points): binary radix tree + depth +
    octree-node map, then the octree; each phase timed with CUDA events (L2
    flushed between repetitions), the oracle on one host thread beside it."""
    import torch
    from del_msh_gb300 import _native
    from del_msh_gb300.QuadOctTree import torch as QOT
    from oracle import build as obuild
    from oracle import oracle as O
    dev = torch.device("cuda", 0)
    _native.load(build_if_missing=True)
    obuild.build_oracle()
    rng = np.random.default_rng(SEED)
    pts = rng.random((2_300_000, 3)).astype(np.float32)
    codes = np.unique(O.vtx2morton(pts, np.eye(4, dtype=np.float32).reshape(-1)))[:2_097_152]
    n = codes.size
    d = torch.from_numpy(codes.view(np.int32)).to(dev).view(torch.uint32)
    flush = torch.empty((L2_FLUSH_BYTES,), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    bn, b2d, b2o, i2b = QOT.bnodes_and_bnode2depth_and_bnode2onode_and_idx2bnode(d, 3)
    num_onode = int(b2o[-1].item()) + 1
    L = _native.load()
    sp = stream.cuda_stream
    scr = torch.empty((L.dm_quad_oct_tree_scratch_bytes(n),), dtype=torch.uint8, device=dev)
    on = torch.full((num_onode, 9), 2 ** 32 - 1, device=dev, dtype=torch.uint32)
    o2d = torch.zeros((num_onode,), device=dev, dtype=torch.uint32)
    o2c = torch.empty((num_onode, 3), device=dev)
    i2o = torch.empty((n,), device=dev, dtype=torch.uint32)
    i2c = torch.empty((n, 3), device=dev)

    def phase1():
        _native.call("dm_quad_oct_tree_bnodes_and_bnode2depth_and_bnode2onode_and_idx2bnode", sp, n, d.data_ptr(), 3,
                     10, bn.data_ptr(), b2d.data_ptr(), b2o.data_ptr(), i2b.data_ptr(), scr.data_ptr(), scr.numel())

    def phase2():
        _native.call("dm_quad_oct_tree_make_tree_from_binary_radix_tree", sp, n, bn.data_ptr(), b2o.data_ptr(),
                     b2d.data_ptr(), i2b.data_ptr(), d.data_ptr(), 3, 10, num_onode, on.data_ptr(), o2d.data_ptr(),
                     o2c.data_ptr(), i2o.data_ptr(), i2c.data_ptr())

    res = {}
    for name, fn in (("binary_tree_and_map", phase1), ("octree", phase2)):
        for _ in range(max(args.warmup, 3)):
            fn()
        times = []
        for _ in range(args.steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
        res[name] = {"ms": statistics.median(times)}
    total = res["binary_tree_and_map"]["ms"] + res["octree"]["ms"]
    line = {"metric": "points/s (quad/oct-tree from sorted unique Morton codes)", "unit": "points/s",
            "value": n / (total * 1e-3), "steps": args.steps,
            "config": {"workload": f"{n} unique 30-bit codes of uniform random 3-D points", "num_onode": num_onode,
                       "l2": "flushed between repetitions"},
            "phases": res, "device_status": _native.device_status(clear=True)}
    if not args.no_cpu:
        t0 = time.perf_counter()
        O.quad_oct_tree(codes, 3)
        t_cpu = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": n / t_cpu, "unit": "points/s", "cores": 1, "kind": "port",
                                "sample": "one full construction (1 thread)"}
    print(json.dumps(line), flush=True)
    return 0


def run_selfx(args):
    """Self-intersection through the BVH: two copies of a displaced torus
    (724x724 grid each, 2,096,704 triangles in all), the second shifted so
    that the two interpenetrate; the LBVH of both is built first, then the
    query is timed with CUDA events (L2 flushed between repetitions), with the
    oracle's recursive search on one host thread beside it."""
    import torch
    from del_msh_gb300 import _native
    from del_msh_gb300 import workloads as W
    from del_msh_gb300.TriMesh3 import torch as TriMesh3
    dev = torch.device("cuda", 0)
    _native.load(build_if_missing=True)
    t, v = W.displaced_torus(724, seed=SEED)
    tri = np.concatenate([t, t + v.shape[0]]).astype(np.uint32)
    vtx = np.concatenate([v, v + np.array([0.35, 0.2, 0.1], np.float32)]).astype(np.float32)
    T, V = tri.shape[0], vtx.shape[0]
    d_tri = torch.from_numpy(tri.view(np.int32)).to(dev).view(torch.uint32)
    d_vtx = torch.from_numpy(vtx).to(dev)
    bvh, aabb = TriMesh3.make_bvhnodes_bvhnode2aabb(d_tri, d_vtx)
    segs, pairs = TriMesh3.self_intersection(d_tri, d_vtx, bvh, aabb)
    cap = max(int(pairs.shape[0]) * 2, 1024)
    out_p = torch.empty((cap, 2), dtype=torch.uint32, device=dev)
    out_s = torch.empty((cap, 2, 3), dtype=torch.float32, device=dev)
    count = torch.zeros((1,), dtype=torch.int32, device=dev)
    flush = torch.empty((L2_FLUSH_BYTES,), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def query():
        _native.call("dm_trimesh3_self_intersection", stream.cuda_stream, T, d_tri.data_ptr(), V, d_vtx.data_ptr(),
                     bvh.data_ptr(), aabb.data_ptr(), cap, out_p.data_ptr(), out_s.data_ptr(), count.data_ptr())

    for _ in range(max(args.warmup, 3)):
        query()
    times = []
    for _ in range(args.steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        query()
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
    ms = statistics.median(times)
    line = {"metric": "triangles/s (self-intersection query through the LBVH)", "unit": "triangles/s",
            "value": T / (ms * 1e-3), "ms": ms, "steps": args.steps,
            "config": {"workload": f"two interpenetrating displaced tori, {T} triangles", "pairs": int(count.item()),
                       "l2": "flushed between repetitions"},
            "device_status": _native.device_status(clear=True)}
    if not args.no_cpu:
        from oracle import build as obuild
        from oracle import oracle as O
        obuild.build_oracle()
        h_bvh, h_aabb = bvh.cpu().numpy(), aabb.cpu().numpy()
        t0 = time.perf_counter()
        rp, _ = O.self_intersection(tri, vtx, h_bvh, h_aabb)
        t_cpu = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": T / t_cpu, "unit": "triangles/s", "cores": 1, "kind": "port",
                                "sample": "one full recursive search (1 thread)", "pairs": int(len(rp))}
    print(json.dumps(line), flush=True)
    return 0


def run_soup(args):
    print(json.dumps(measure_soup(args.steps, args.warmup, cpu=not args.no_cpu)), flush=True)
    return 0


def measure_soup(steps: int, warmup: int, cpu: bool):
    """Adversarial Morton distribution: 4,194,304-triangle soup whose centroids
    come from 32 Gaussian clusters (sigma 1e-3 in the unit cube), so many
    30-bit codes repeat and duplicate runs become long chains in the tree.
    One step = full LBVH build + cast of 1,048,576 rays from uniformly random
    points of the cube boundary in uniformly random inward directions."""
    import torch
    from del_msh_gb300 import _native
    from del_msh_gb300 import workloads as W
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    L = _native.load(build_if_missing=True)
    tri, vtx = W.clustered_soup(4_194_304, seed=SEED)
    org, d = W.cube_boundary_rays(1_048_576, seed=SEED)
    T, V, R = tri.shape[0], vtx.shape[0], org.shape[0]
    d_tri = torch.from_numpy(tri.view(np.int32)).to(dev)
    d_vtx = torch.from_numpy(vtx).to(dev)
    d_org, d_dir = torch.from_numpy(org).to(dev), torch.from_numpy(d).to(dev)
    bvh = torch.empty((2 * T - 1, 3), dtype=torch.int32, device=dev)
    aabb = torch.empty((2 * T - 1, 6), dtype=torch.float32, device=dev)
    hit = torch.empty((R,), dtype=torch.int32, device=dev)
    ht = torch.empty((R,), dtype=torch.float32, device=dev)
    height = torch.zeros((1,), dtype=torch.int32, device=dev)
    bs, cs = L.dm_trimesh3_build_scratch_bytes(T), L.dm_cast_scratch_bytes(R, T)
    b_scr = torch.empty((bs,), dtype=torch.uint8, device=dev)
    c_scr = torch.empty((cs,), dtype=torch.uint8, device=dev)
    flush = torch.empty((L2_FLUSH_BYTES,), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream

    def build(want_height=False):
        # the height (reported once, untimed) needs the tree-order climb
        _native.call("dm_trimesh3_build_ex", sp, T, d_tri.data_ptr(), V, d_vtx.data_ptr(), bvh.data_ptr(),
                     aabb.data_ptr(), None, None, None, None, height.data_ptr() if want_height else None,
                     b_scr.data_ptr(), bs)

    def cast():
        _native.call("dm_search_bvh3_first_intersection_ray", sp, R, d_org.data_ptr(), d_dir.data_ptr(),
                     hit.data_ptr(), ht.data_ptr(), None, T, d_tri.data_ptr(), V, d_vtx.data_ptr(), bvh.data_ptr(),
                     aabb.data_ptr(), c_scr.data_ptr(), cs)

    build(want_height=True)
    for _ in range(max(warmup, 3)):
        build()
        cast()
    torch.cuda.synchronize()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
    for k in range(steps):
        flush.zero_()
        ev[k][0].record(stream)
        build()
        ev[k][1].record(stream)
        cast()
        ev[k][2].record(stream)
    torch.cuda.synchronize()
    b_ms = statistics.mean(e[0].elapsed_time(e[1]) for e in ev)
    c_ms = statistics.mean(e[1].elapsed_time(e[2]) for e in ev)
    stage = (ctypes.c_float * 4)()
    runs = []
    for _ in range(5):
        _native.call("dm_trimesh3_build_profiled", sp, T, d_tri.data_ptr(), V, d_vtx.data_ptr(), bvh.data_ptr(),
                     aabb.data_ptr(), b_scr.data_ptr(), bs, ctypes.cast(stage, ctypes.c_void_p))
        runs.append(list(stage))
    peak, _ = peaks()
    nb = algorithmic_bytes(T, V, R)
    line = {"metric": "rays/s (adversarial soup: build + cast per step)", "unit": UNIT,
            "value": R / ((b_ms + c_ms) * 1e-3), "ms_per_step": b_ms + c_ms, "steps": steps,
            "config": {"workload": "4,194,304-triangle soup in 32 Gaussian clusters (sigma 1e-3), 1,048,576 "
                                   "cube-boundary rays", "num_tri": T, "num_vtx": V, "rays": R,
                       "tree_height": int(height.item()), "l2": "flushed between timed steps"},
            "build_ms": b_ms, "cast_ms": c_ms, "build_tris_per_s": T / (b_ms * 1e-3),
            "cast_rays_per_s": R / (c_ms * 1e-3),
            "stage_ms": {k: statistics.mean(r[i] for r in runs)
                         for i, k in enumerate(("morton", "sort", "topology", "refit"))},
            "build_roofline_frac": nb["build"] / (b_ms * 1e-3) / 1e9 / peak,
            "hits": int((hit != -1).sum().item()), "device_status": _native.device_status(clear=True)}
    if cpu:
        from oracle import build as obuild
        from oracle import oracle as O
        obuild.build_oracle()
        t0 = time.perf_counter()
        r = O.build(tri, vtx)
        t1 = time.perf_counter()
        O.cast_rays(org, d, tri, vtx, r["bvhnodes"], r["bvhnode2aabb"])
        t2 = time.perf_counter()
        line["cpu_baseline"] = {"build_s": t1 - t0, "cast_s": t2 - t1, "cores": O.default_threads(), "kind": "port",
                                "value": R / (t2 - t0), "unit": UNIT}
    del d_tri, d_vtx, d_org, d_dir, bvh, aabb, hit, ht, b_scr, c_scr, flush
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return line


def read_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary
    (profiles/ncu_torus2m_step.md lines `traffic <kernel> <bytes>`), else None."""
    p = ROOT / "profiles" / "ncu_torus2m_step.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        parts = line.strip().strip("`").split()
        if len(parts) == 3 and parts[0] == "traffic" and parts[1] == kernel:
            return float(parts[2])
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batched / served / soup keys of the default line")
    ap.add_argument("--workload", choices=["single", "batched", "served", "soup", "render", "octree", "selfx"],
                    default="single")
    ap.add_argument("--num-mesh", type=int, default=4096, help="meshes of the batched workload")
    ap.add_argument("--pool", type=int, default=512, help="meshes of the served pool")
    ap.add_argument("--requests", type=int, default=1000, help="requests per served trace")
    ap.add_argument("--slots", type=int, default=8, help="concurrent request slots of the server")
    ap.add_argument("--budget-gb", type=float, default=120.0, help="HBM budget of the server")
    ap.add_argument("--loads", type=float, nargs="*", default=[0.5, 0.8, 2.0, 4.0],
                    help="offered loads as fractions of the plain path's capacity")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "served":
        return run_served(args)
    if args.workload == "soup":
        return run_soup(args)
    if args.workload == "render":
        return run_render(args)
    if args.workload == "octree":
        return run_octree(args)
    if args.workload == "selfx":
        return run_selfx(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
