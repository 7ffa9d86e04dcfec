"""Autotuner for the launch parameters of ``dm_tuning`` (include/delmsh_gb300.h).

The choices it sweeps are compiled into the library:

- the persistent cast's block size and on-chip stack depth (frames per ray
  before the overflow tiers), as (threads, frames) pairs;
- the pixel tile of one warp (tile_w x 32/tile_w);
- the radix sort's look-back window (predecessor tiles read per round);
- the phase minima of the persistent cast (how many lanes of a warp must
  wait to take new rays, to test a triangle, or to pop frames before the
  warp runs that phase), swept at the fastest cast shape.

Every choice gives the same results, and the sweep checks that: each
candidate's output must equal the default's bit for bit, or the candidate is
rejected.  Timing uses CUDA events on the launching stream, with the L2
flushed (a 256 MiB write) outside the timed region between repetitions.

``tune()`` writes the fastest choice, with the whole sweep, to a JSON table;
``apply()`` sets it when the table was measured on a device of the same name.
``del_msh_gb300._native.load()`` calls ``apply()`` on the table shipped next to
this file, if there is one.

``tune_build()`` sweeps the single-mesh build by size class (a displaced
torus standing for each class): the cooperative front or the separate
kernels, for the separate kernels the radix width (three 10-bit or four 8-bit
passes), and the topology kernel's block size; ``tune_batched()`` sweeps the
batched build's path (on chip or the global sort) and least cluster size on
the ragged 4096-mesh workload and on a batch of meshes of up to 16384
triangles.  ``tune_all()`` runs the three and writes one table.
"""
from __future__ import annotations

import json
import pathlib
import statistics
import time

from . import _native

DEFAULT_TABLE = pathlib.Path(__file__).resolve().parent / "tuning.json"
CAST_CHOICES = [(128, 64), (64, 64), (256, 64), (128, 32), (128, 96)]
TILE_CHOICES = [4, 8, 16, 32]
SORT_WINDOWS = [4, 8]
PHASE_CHOICES = [(1, 1, 1), (4, 4, 4), (6, 6, 6), (8, 8, 8), (8, 6, 6), (12, 8, 8), (16, 8, 8), (12, 12, 12),
                 (16, 12, 12), (24, 8, 8), (20, 10, 10), (8, 4, 4), (12, 4, 4), (12, 6, 6), (16, 6, 6), (6, 2, 2)]
DEFAULT = dict(cast_threads=128, cast_stack=64, tile_w=8, sort_window=4, cast_refill_min=6, cast_leaf_min=6,
               cast_ascend_min=6, cast_long_steps=64, batch_path=0, batch_cluster=0)
_PHASE_KEYS = ("cast_refill_min", "cast_leaf_min", "cast_ascend_min")


def _device_name(device) -> str | None:
    try:
        import torch
        if not torch.cuda.is_available():
            return None
        return torch.cuda.get_device_name(torch.device(device))
    except Exception:  # no torch / no driver: nothing to match against
        return None


def apply(path=DEFAULT_TABLE, device="cuda:0") -> dict | None:
    """Sets the table's best choice if it was measured on this device model;
    returns it (or None when nothing was applied)."""
    p = pathlib.Path(path)
    if not p.exists():
        return None
    table = json.loads(p.read_text())
    name = _device_name(device)
    if name is None or table.get("device") != name:
        return None
    best = dict(table["best"])
    batched = table.get("batched_best", {})
    _native.set_tuning(best["cast_threads"], best["cast_stack"], best["tile_w"], best["sort_window"],
                       *(best.get(k, 0) for k in _PHASE_KEYS),  # 0: the library default
                       0, batched.get("batch_path", 0), batched.get("batch_cluster", 0))
    if "build_classes" in table:
        _native.set_build_classes([{k: c[k] for k in ("max_tri", "build_path", "sort_radix", "topo_threads")}
                                   for c in table["build_classes"]])
    best.update(batched)
    return best


def pick_cast(cast_sweep, tolerance: float = 0.01) -> dict:
    """The cast shape to use: among the identical-output choices within
    `tolerance` of the fastest, the one with the deepest on-chip stack (fewer
    rays of deep trees fall back to the global-memory tiers, which this
    workload does not exercise), then the fastest."""
    ok = [c for c in cast_sweep if c["identical"]]
    fastest = min(c["ms"] for c in ok)
    near = [c for c in ok if c["ms"] <= fastest * (1 + tolerance)]
    return min(near, key=lambda c: (-c["cast_stack"], c["ms"]))


def pick_over_default(sweep, is_default, key="ms", tolerance: float = 0.01) -> dict:
    """The default choice unless an identical-output choice is more than
    `tolerance` faster; then the fastest."""
    ok = [c for c in sweep if c["identical"]]
    dflt = next(c for c in ok if is_default(c))
    fastest = min(ok, key=lambda c: c[key])
    return fastest if fastest[key] < dflt[key] * (1 - tolerance) else dflt


def _events_ms(torch, stream, fn, flush, reps: int) -> float:
    times = []
    for _ in range(reps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
    return statistics.median(times)


def tune(device="cuda:0", out=DEFAULT_TABLE, reps: int = 15, ndiv: int = 1024, img=(1920, 1080),
         seed: int = 0) -> dict:
    """Sweeps every compiled choice on the single-mesh workload (a displaced
    torus on an ndiv x ndiv grid, a pinhole image of img pixels), writes the
    table to `out` (unless None) and applies its best choice."""
    import numpy as np
    import torch

    from . import workloads as W

    dev = torch.device(device)
    L = _native.load()
    tri, vtx = W.displaced_torus(ndiv, seed=seed)
    eye = W.random_viewpoint(3.0, seed=seed)
    m = W.pinhole_ndc2world(eye, aspect=img[0] / img[1])  # column-major, as the C ABI reads it
    T, V = tri.shape[0], vtx.shape[0]
    d_tri = torch.from_numpy(tri.view(np.int32)).to(dev).view(torch.uint32)
    d_vtx = torch.from_numpy(vtx).to(dev)
    d_m = torch.from_numpy(m).to(dev)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    flush = torch.empty((256 << 20,), dtype=torch.uint8, device=dev)
    bvh = torch.empty((2 * T - 1, 3), dtype=torch.int32, device=dev)
    aabb = torch.empty((2 * T - 1, 6), dtype=torch.float32, device=dev)
    p2t = torch.empty((img[1], img[0]), dtype=torch.int32, device=dev)
    tt = torch.empty((img[1], img[0]), dtype=torch.float32, device=dev)
    bs, cs = L.dm_trimesh3_build_scratch_bytes(T), L.dm_cast_scratch_bytes(img[0] * img[1], T)
    b_scr = torch.empty((bs,), dtype=torch.uint8, device=dev)
    c_scr = torch.empty((cs,), dtype=torch.uint8, device=dev)

    def build():
        _native.call("dm_trimesh3_make_bvhnodes_bvhnode2aabb", sp, T, d_tri.data_ptr(), V, d_vtx.data_ptr(),
                     bvh.data_ptr(), aabb.data_ptr(), b_scr.data_ptr(), bs)

    def cast():
        _native.call("dm_pix2tri_by_raycast", sp, img[0], img[1], p2t.data_ptr(), tt.data_ptr(), T,
                     d_tri.data_ptr(), V, d_vtx.data_ptr(), bvh.data_ptr(), aabb.data_ptr(), d_m.data_ptr(),
                     c_scr.data_ptr(), cs)

    start = time.time()
    _native.set_tuning(**DEFAULT)
    build()
    cast()
    torch.cuda.synchronize(dev)
    ref_tree = (bvh.clone(), aabb.clone())
    ref_img = (p2t.clone(), tt.clone().view(torch.int32))

    def same_tree():
        return bool(torch.equal(bvh, ref_tree[0]) and torch.equal(aabb.view(torch.int32), ref_tree[1].view(torch.int32)))

    def same_img():
        return bool(torch.equal(p2t, ref_img[0]) and torch.equal(tt.view(torch.int32), ref_img[1]))

    sweep = {"cast": [], "sort": [], "phase": []}
    phase0 = tuple(DEFAULT[k] for k in _PHASE_KEYS)
    for threads, frames in CAST_CHOICES:
        for tile_w in TILE_CHOICES:
            _native.set_tuning(threads, frames, tile_w, DEFAULT["sort_window"], *phase0)
            for _ in range(3):
                cast()
            ms = _events_ms(torch, stream, cast, flush, reps)
            sweep["cast"].append(dict(cast_threads=threads, cast_stack=frames, tile_w=tile_w, ms=ms,
                                      identical=same_img()))
    for window in SORT_WINDOWS:
        _native.set_tuning(DEFAULT["cast_threads"], DEFAULT["cast_stack"], DEFAULT["tile_w"], window, *phase0)
        for _ in range(3):
            build()
        ms = _events_ms(torch, stream, build, flush, reps)
        sweep["sort"].append(dict(sort_window=window, build_ms=ms, identical=same_tree()))
    bc = pick_cast(sweep["cast"])
    for mins in PHASE_CHOICES:
        _native.set_tuning(bc["cast_threads"], bc["cast_stack"], bc["tile_w"], DEFAULT["sort_window"], *mins)
        for _ in range(3):
            cast()
        ms = _events_ms(torch, stream, cast, flush, reps)
        sweep["phase"].append(dict(zip(_PHASE_KEYS, mins), ms=ms, identical=same_img()))
    status = _native.device_status(clear=True)

    ok_sort = [c for c in sweep["sort"] if c["identical"]]
    ok_phase = [c for c in sweep["phase"] if c["identical"]]
    bsrt = min(ok_sort, key=lambda c: c["build_ms"])
    bph = min(ok_phase, key=lambda c: c["ms"])
    best = dict(cast_threads=bc["cast_threads"], cast_stack=bc["cast_stack"], tile_w=bc["tile_w"],
                sort_window=bsrt["sort_window"], **{k: bph[k] for k in _PHASE_KEYS})
    table = {
        "device": torch.cuda.get_device_name(dev),
        "sm_count": torch.cuda.get_device_properties(dev).multi_processor_count,
        "torch": torch.__version__,
        "cuda": torch.version.cuda,
        "library": L.dm_version().decode(),
        "workload": f"displaced torus {ndiv}x{ndiv} grid ({T} tris), {img[0]}x{img[1]} pinhole cast, seed {seed}",
        "timing": f"median of {reps} CUDA-event timings per choice, L2 flushed between them",
        "default": DEFAULT,
        "best": best,
        "speedup_cast_vs_default": next(c["ms"] for c in sweep["cast"]
                                        if c["cast_threads"] == DEFAULT["cast_threads"]
                                        and c["cast_stack"] == DEFAULT["cast_stack"]
                                        and c["tile_w"] == DEFAULT["tile_w"]) / min(bc["ms"], bph["ms"]),
        "speedup_phase_vs_any_lane": next(c["ms"] for c in sweep["phase"]
                                          if all(c[k] == 1 for k in _PHASE_KEYS)) / bph["ms"],
        "rejected": [c for c in sweep["cast"] + sweep["sort"] + sweep["phase"] if not c["identical"]],
        "device_status": status,
        "sweep": sweep,
        "sweep_s": time.time() - start,
    }
    _native.set_tuning(**best)
    if out is not None:
        pathlib.Path(out).write_text(json.dumps(table, indent=1) + "\n")
    return table


BUILD_CLASSES = [(131_072, 181), (1_048_576, 512), (4_194_304, 1024), (0xFFFFFFFF, 2048)]  # (bound, torus ndiv)
BUILD_CHOICES = ([dict(build_path=0, sort_radix=0, topo_threads=t) for t in (128, 256, 512)] +
                 [dict(build_path=1, sort_radix=r, topo_threads=t) for r in (8, 10) for t in (128, 256, 512)])
BATCH_CHOICES = [dict(batch_path=0, batch_cluster=0), dict(batch_path=0, batch_cluster=2),
                 dict(batch_path=0, batch_cluster=4), dict(batch_path=1, batch_cluster=0)]


def tune_build(device="cuda:0", reps: int = 15, classes=BUILD_CLASSES, seed: int = 0) -> list:
    """Per size class, every build choice on a displaced torus of that class:
    build time (median, L2 flushed) and whether the tree and boxes equal the
    default choice's bit for bit.  Returns the table's class entries, each
    with its fastest identical choice and its sweep."""
    import numpy as np
    import torch

    from . import workloads as W

    dev = torch.device(device)
    L = _native.load()
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    flush = torch.empty((256 << 20,), dtype=torch.uint8, device=dev)
    before = _native.get_build_classes()
    out = []
    try:
        for bound, ndiv in classes:
            tri, vtx = W.displaced_torus(ndiv, seed=seed)
            T, V = tri.shape[0], vtx.shape[0]
            d_tri = torch.from_numpy(tri.view(np.int32)).to(dev)
            d_vtx = torch.from_numpy(vtx).to(dev)
            bvh = torch.empty((2 * T - 1, 3), dtype=torch.int32, device=dev)
            aabb = torch.empty((2 * T - 1, 6), dtype=torch.float32, device=dev)
            bs = L.dm_trimesh3_build_scratch_bytes(T)
            scr = torch.empty((bs,), dtype=torch.uint8, device=dev)

            def build():
                _native.call("dm_trimesh3_make_bvhnodes_bvhnode2aabb", sp, T, d_tri.data_ptr(), V,
                             d_vtx.data_ptr(), bvh.data_ptr(), aabb.data_ptr(), scr.data_ptr(), bs)

            _native.set_build_classes([])
            build()
            torch.cuda.synchronize(dev)
            ref = (bvh.clone(), aabb.clone().view(torch.int32))
            sweep = []
            for c in BUILD_CHOICES:
                _native.set_build_classes([dict(max_tri=0xFFFFFFFF, **c)])
                for _ in range(3):
                    build()
                ms = _events_ms(torch, stream, build, flush, reps)
                same = bool(torch.equal(bvh, ref[0]) and torch.equal(aabb.view(torch.int32), ref[1]))
                sweep.append(dict(c, ms=ms, identical=same))
            best = pick_over_default(sweep, lambda c: c["build_path"] == 0 and c["topo_threads"] == 256)
            out.append(dict(max_tri=bound, build_path=best["build_path"], sort_radix=best["sort_radix"],
                            topo_threads=best["topo_threads"], ms=best["ms"], workload_tri=T, sweep=sweep))
            del d_tri, d_vtx, bvh, aabb, scr
            torch.cuda.empty_cache()
    finally:
        _native.set_build_classes(before)
    return out


def tune_batched(device="cuda:0", reps: int = 5, seed: int = 0) -> list:
    """The batched build's choices on the ragged 4096-mesh workload (triangle
    counts log-uniform in [64, 65536]) and on 4096 meshes of [64, 16384]
    triangles: build time of MeshBatch.build (median, L2 flushed) and whether
    every tree and box equals the default's bit for bit."""
    import torch

    from . import workloads as W
    from .batch import MeshBatch

    dev = torch.device(device)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty((256 << 20,), dtype=torch.uint8, device=dev)
    base = _native.get_tuning()
    out = []
    try:
        for tmax in (65536, 16384):
            meshes = W.ragged_batch(num_mesh=4096, tmin=64, tmax=tmax, seed=seed)
            b = MeshBatch(meshes, dev)
            _native.set_tuning(**dict(base, batch_path=0, batch_cluster=0))
            b.build()
            torch.cuda.synchronize(dev)
            ref = (b.bvhnodes.clone().view(torch.int32), b.bvhnode2aabb.clone().view(torch.int32))
            sweep = []
            for c in BATCH_CHOICES:
                _native.set_tuning(**dict(base, **c))
                for _ in range(2):
                    b.build()
                ms = _events_ms(torch, stream, b.build, flush, reps)
                same = bool(torch.equal(b.bvhnodes.view(torch.int32), ref[0]) and
                            torch.equal(b.bvhnode2aabb.view(torch.int32), ref[1]))
                sweep.append(dict(c, ms=ms, identical=same))
            best = pick_over_default(sweep, lambda c: c["batch_path"] == 0 and c["batch_cluster"] == 0)
            out.append(dict(max_tri=b.max_tri, total_tri=b.total_tri, batch_path=best["batch_path"],
                            batch_cluster=best["batch_cluster"], ms=best["ms"], sweep=sweep))
            del b
            torch.cuda.empty_cache()
    finally:
        _native.set_tuning(**base)
    return out


def tune_all(device="cuda:0", out=DEFAULT_TABLE, reps: int = 15) -> dict:
    """tune() (cast and look-back window on the single-mesh workload), then
    tune_build() and tune_batched(); one table with all three.  The batched
    choice applied is the one measured on the ragged 4096-mesh workload."""
    table = tune(device, None, reps)
    start = time.time()
    table["build_classes"] = tune_build(device, reps)
    table["batched"] = tune_batched(device)
    big = table["batched"][0]
    table["batched_best"] = {"batch_path": big["batch_path"], "batch_cluster": big["batch_cluster"]}
    table["device_status"] = max(table["device_status"], _native.device_status(clear=True))
    table["sweep_s"] += time.time() - start
    if out is not None:
        pathlib.Path(out).write_text(json.dumps(table, indent=1) + "\n")
        apply(out)
    return table


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--device", default="cuda:0")
    ap.add_argument("--out", default=str(DEFAULT_TABLE))
    ap.add_argument("--reps", type=int, default=15)
    args = ap.parse_args()
    t = tune_all(args.device, args.out, args.reps)
    print(json.dumps({"device": t["device"], "best": t["best"], "batched_best": t["batched_best"],
                      "build_classes": [{k: c[k] for k in ("max_tri", "build_path", "sort_radix", "topo_threads",
                                                          "ms")} for c in t["build_classes"]],
                      "sweep_s": t["sweep_s"]}))
