"""Multi-GPU partitions of the path, checked on the CPU with two gloo ranks.

Each rank takes its share (meshes by id for a batch; a pixel range for one
mesh's cast), computes it (here with the oracle, standing in for the rank's
GPU), and the outputs gathered on rank 0 in global order must equal the
single-rank result.  The gather is the host's collection of results; no
collective runs on the data path."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _paths():
    for p in (ROOT, os.path.join(ROOT, "del-msh_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _batch():
    _paths()
    from del_msh_gb300 import workloads as W
    return W.ragged_batch(num_mesh=12, tmin=64, tmax=3000, seed=11)


def _mesh_result(O, tri, vtx):
    from del_msh_gb300 import workloads as W
    r = O.build(tri, vtx)
    tf = W.box_ortho_ndc2world(vtx.min(0), vtx.max(0))
    p2t, tt = O.pix2tri(tri, vtx, r["bvhnodes"], r["bvhnode2aabb"], tf, 24, 16, threads=1)
    return r["bvhnodes"], r["bvhnode2aabb"].view(np.uint32), p2t, tt.view(np.uint32)


def _single_mesh():
    _paths()
    from del_msh_gb300 import workloads as W
    tri, vtx = W.jittered_icosphere(3, seed=4)
    return tri, vtx, W.ortho_ndc2world(), 40, 30


def _rank_main(rank, world, port, out):
    _paths()
    import torch.distributed as dist
    from oracle import build as obuild
    from oracle import oracle as O
    from del_msh_gb300 import partition as P
    obuild.build_oracle()
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # meshes by id
    meshes = _batch()
    ids = P.partition_meshes([t.shape[0] for t, _ in meshes], world)[rank]
    mine = (ids.tolist(), [_mesh_result(O, *meshes[m]) for m in ids])
    # one mesh's pixels, tree replicated
    tri, vtx, tf, w, h = _single_mesh()
    r = O.build(tri, vtx)
    first, last = P.shard_pixels(w * h, world, rank)
    rays = [O.ray_for_pixel(i, w, h, tf) for i in range(first, last)]
    org = np.array([o for o, _ in rays], np.float32).reshape(-1, 3)
    d = np.array([x for _, x in rays], np.float32).reshape(-1, 3)
    hit, t = O.cast_rays(org, d, tri, vtx, r["bvhnodes"], r["bvhnode2aabb"], threads=1)
    pix = ((first, last), np.stack([hit, t.view(np.uint32)], 1))
    gathered = [None] * world
    dist.all_gather_object(gathered, (mine, pix))
    if rank == 0:
        out.put(gathered)
    dist.barrier()
    dist.destroy_process_group()


def test_partition_is_a_balanced_disjoint_cover():
    _paths()
    from del_msh_gb300 import partition as P
    rng = np.random.default_rng(0)
    counts = np.exp(rng.uniform(np.log(64), np.log(65536), 4096)).astype(np.int64)
    for world in (1, 2, 3, 8):
        parts = P.partition_meshes(counts, world)
        allid = np.concatenate(parts)
        assert np.array_equal(np.sort(allid), np.arange(counts.size))
        loads = np.array([counts[p].sum() for p in parts])
        assert loads.max() - loads.min() <= counts.max()
        assert all((np.diff(p) > 0).all() for p in parts)
    for world in (1, 2, 5):
        spans = [P.shard_pixels(1000, world, r) for r in range(world)]
        assert spans[0][0] == 0 and spans[-1][1] == 1000
        assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
    with pytest.raises(ValueError):
        P.gather_meshes([([0], ["a"]), ([0], ["b"])], 1)


def test_two_gloo_ranks_equal_one_rank(oracle):
    import torch.multiprocessing as mp
    _paths()
    from del_msh_gb300 import partition as P
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    gathered = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    meshes = _batch()
    got = P.gather_meshes([g[0] for g in gathered], len(meshes))
    assert all(len(g[0][0]) > 0 for g in gathered)  # both ranks had work
    for m, (tri, vtx) in enumerate(meshes):
        want = _mesh_result(oracle, tri, vtx)
        for a, b in zip(got[m], want):
            assert np.array_equal(a, b), m
    tri, vtx, tf, w, h = _single_mesh()
    img = P.gather_pixels([g[1] for g in gathered], w * h)
    r = oracle.build(tri, vtx)
    p2t, tt = oracle.pix2tri(tri, vtx, r["bvhnodes"], r["bvhnode2aabb"], tf, w, h, threads=1)
    assert np.array_equal(img[:, 0], p2t.reshape(-1))
    assert np.array_equal(img[:, 1], tt.reshape(-1).view(np.uint32))
