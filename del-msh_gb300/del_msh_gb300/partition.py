"""Work partitions for running the path on several GPUs, one process per GPU.

The units of this path are independent, so no partition needs a collective
on the data path (there is no reference counterpart: del-msh runs on one
device):

* **Meshes of a batch or a served pool** are split by mesh id
  (``partition_meshes``): each rank builds, keeps resident and casts only its
  own meshes with a ``MeshBatch`` (or its own server), and each mesh's
  results are those of the single-rank run, since a mesh's tree and image
  depend on that mesh alone.  Ranks are balanced by triangle count
  (largest-first onto the least-loaded rank).
* **The rays of one single-mesh cast** are split into contiguous pixel ranges
  (``shard_pixels``): every rank builds (or receives) the same tree and
  casts its range with ``dm_search_bvh3_first_intersection_ray``.
* ``gather_meshes`` / ``gather_pixels`` put the per-rank outputs back in
  global order on the host, which is where a caller would collect them.
"""
from __future__ import annotations

import numpy as np


def partition_meshes(tri_counts, world: int):
    """Mesh ids of each of `world` ranks: a disjoint cover of range(len(tri_counts)),
    each rank's ids ascending.  Meshes are placed largest first on the rank
    with the fewest triangles so far (ties to the lower rank, then the lower
    mesh id), so every rank's share is within one mesh of the mean."""
    counts = np.asarray(tri_counts, np.int64)
    if world < 1:
        raise ValueError("world must be >= 1")
    if (counts < 1).any():
        raise ValueError("every mesh needs at least one triangle")
    order = np.lexsort((np.arange(counts.size), -counts))  # size descending, id ascending
    load = np.zeros(world, np.int64)
    owner = np.empty(counts.size, np.int64)
    for m in order:
        r = int(np.argmin(load))  # argmin returns the lowest rank on ties
        owner[m] = r
        load[r] += counts[m]
    return [np.flatnonzero(owner == r).astype(np.int64) for r in range(world)]


def shard_pixels(num_pixel: int, world: int, rank: int):
    """[first, last) pixel range of `rank`: contiguous, sizes differing by at most one."""
    if not 0 <= rank < world:
        raise ValueError("rank outside 0..world-1")
    base, extra = divmod(int(num_pixel), world)
    first = rank * base + min(rank, extra)
    return first, first + base + (1 if rank < extra else 0)


def gather_meshes(parts, num_mesh: int):
    """Per-mesh outputs in global mesh order from [(ids, outputs), ...] of the
    ranks, where outputs[k] belongs to mesh ids[k]."""
    out = [None] * num_mesh
    for ids, outputs in parts:
        for m, o in zip(ids, outputs):
            if out[int(m)] is not None:
                raise ValueError(f"mesh {int(m)} came from two ranks")
            out[int(m)] = o
    missing = [m for m, o in enumerate(out) if o is None]
    if missing:
        raise ValueError(f"meshes {missing[:8]} came from no rank")
    return out


def gather_pixels(parts, num_pixel: int):
    """The whole image (flat) from [((first, last), values), ...] of the ranks."""
    parts = sorted(parts, key=lambda p: p[0][0])
    pos = 0
    for (first, last), values in parts:
        if first != pos or len(values) != last - first:
            raise ValueError("pixel ranges do not tile the image")
        pos = last
    if pos != num_pixel:
        raise ValueError("pixel ranges do not cover the image")
    return np.concatenate([np.asarray(v) for _, v in parts])
