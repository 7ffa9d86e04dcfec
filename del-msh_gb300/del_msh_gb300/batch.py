"""Batches of independent triangle meshes of uneven sizes, resident on one GPU.

A ``MeshBatch`` stores its meshes back to back and builds / casts all of them
with one launch sequence each (``dm_batch_trimesh3_build`` and
``dm_batch_pix2tri_by_raycast``); ``capture`` records build + cast into a CUDA
graph that ``replay`` relaunches with one call.  Every mesh's slice of the
results is bit for bit the single-mesh result for that mesh (the tests check
it against ``PlainPath``, one launch sequence per mesh, and the oracle).

There is no reference counterpart: del-msh builds and casts one mesh per call
(``TriMesh3/torch.py:233-285``, ``Pix2Tri/torch.py:8-61``); ``PlainPath`` is
that per-mesh usage on the same GPU.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native


def _u32(a: np.ndarray, dev) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint32).view(np.int32)).to(dev).view(torch.uint32)


class MeshBatch:
    """Meshes (a list of (tri2vtx u32[T,3], vtx2xyz f32[V,3]) numpy arrays)
    concatenated on ``device`` with their trees, scratch and casting buffers."""

    def __init__(self, meshes, device="cuda:0", want_heights: bool = False):
        self.device = torch.device(device)
        self.num_mesh = len(meshes)
        assert self.num_mesh >= 1
        tri_counts = np.array([m[0].shape[0] for m in meshes], np.int64)
        vtx_counts = np.array([m[1].shape[0] for m in meshes], np.int64)
        assert (tri_counts >= 1).all(), "every mesh needs at least one triangle"
        assert (vtx_counts >= 1).all()
        self.tri_off = np.concatenate([[0], np.cumsum(tri_counts)]).astype(np.uint32)
        self.vtx_off = np.concatenate([[0], np.cumsum(vtx_counts)]).astype(np.uint32)
        self.total_tri = int(self.tri_off[-1])
        self.total_vtx = int(self.vtx_off[-1])
        self.max_tri = int(tri_counts.max())
        self.node_off = (2 * self.tri_off[:-1].astype(np.int64) - np.arange(self.num_mesh)).astype(np.int64)
        dev = self.device
        self.d_tri_off = _u32(self.tri_off, dev)
        self.d_vtx_off = _u32(self.vtx_off, dev)
        self.tri2vtx = _u32(np.concatenate([m[0].reshape(-1, 3) for m in meshes]), dev)
        self.vtx2xyz = torch.from_numpy(np.concatenate([m[1].reshape(-1, 3) for m in meshes]).astype(np.float32)).to(dev)
        num_node = 2 * self.total_tri - self.num_mesh
        self.bvhnodes = torch.empty((num_node, 3), dtype=torch.uint32, device=dev)
        self.bvhnode2aabb = torch.empty((num_node, 6), dtype=torch.float32, device=dev)
        # per-mesh tree heights, only on request: they come from the tree-order
        # climb, which is slower than the range-query refit
        self.heights = torch.zeros((self.num_mesh,), dtype=torch.int32, device=dev) if want_heights else None
        L = _native.load()
        self._build_bytes = L.dm_batch_build_scratch_bytes(self.num_mesh, self.total_tri)
        self._build_scratch = torch.empty((self._build_bytes,), dtype=torch.uint8, device=dev)
        self._cast_bytes = 0
        self._cast_scratch = None
        self.graph = None

    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def build(self):
        """Builds every mesh's LBVH (asynchronous on the current stream)."""
        _native.call("dm_batch_trimesh3_build", self._stream(), self.num_mesh, self.d_tri_off.data_ptr(),
                     self.d_vtx_off.data_ptr(), self.total_tri, self.total_vtx, self.max_tri, self.tri2vtx.data_ptr(),
                     self.vtx2xyz.data_ptr(), self.bvhnodes.data_ptr(), self.bvhnode2aabb.data_ptr(),
                     self.heights.data_ptr() if self.heights is not None else None, self._build_scratch.data_ptr(),
                     self._build_bytes)

    def alloc_cast(self, img_w: int, img_h: int, want_t: bool = True):
        """Output images (num_mesh, img_h, img_w) and cast scratch for img_w x img_h per mesh."""
        n = self.num_mesh * img_w * img_h
        self.img_w, self.img_h = img_w, img_h
        self.pix2tri = torch.empty((self.num_mesh, img_h, img_w), dtype=torch.uint32, device=self.device)
        self.pix2t = torch.empty((self.num_mesh, img_h, img_w), dtype=torch.float32, device=self.device) \
            if want_t else None
        need = _native.load().dm_batch_cast_scratch_bytes(n, self.max_tri)
        if need > self._cast_bytes:
            self._cast_scratch = torch.empty((need,), dtype=torch.uint8, device=self.device)
            self._cast_bytes = need

    def cast_pixels(self, transforms_colmajor: torch.Tensor):
        """Casts every mesh's image; transforms_colmajor: (num_mesh, 16) float32
        column-major ndc->world on the device.  Returns (pix2tri, pix2t)."""
        assert transforms_colmajor.shape == (self.num_mesh, 16) and transforms_colmajor.dtype == torch.float32
        assert transforms_colmajor.is_contiguous() and transforms_colmajor.device == self.device
        _native.call("dm_batch_pix2tri_by_raycast", self._stream(), self.num_mesh, self.d_tri_off.data_ptr(),
                     self.d_vtx_off.data_ptr(), self.total_tri, self.total_vtx, self.max_tri,
                     self.tri2vtx.data_ptr(), self.vtx2xyz.data_ptr(), self.bvhnodes.data_ptr(),
                     self.bvhnode2aabb.data_ptr(), self.img_w, self.img_h, transforms_colmajor.data_ptr(),
                     self.pix2tri.data_ptr(), None if self.pix2t is None else self.pix2t.data_ptr(),
                     self._cast_scratch.data_ptr(), self._cast_bytes)
        return self.pix2tri, self.pix2t

    def capture(self, transforms_colmajor: torch.Tensor):
        """Records build + cast into a CUDA graph (alloc_cast first).  The
        graph reads the current contents of vtx2xyz / transforms at replay."""
        self._graph_transforms = transforms_colmajor
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self.build()
            self.cast_pixels(transforms_colmajor)
        torch.cuda.current_stream(self.device).wait_stream(s)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.build()
            self.cast_pixels(transforms_colmajor)
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()

    def mesh_tree(self, m: int):
        """(bvhnodes, bvhnode2aabb) slice of mesh m (mesh-local indices)."""
        a = int(self.node_off[m])
        b = a + 2 * int(self.tri_off[m + 1] - self.tri_off[m]) - 1
        return self.bvhnodes[a:b], self.bvhnode2aabb[a:b]


class PlainPath:
    """The same meshes built and cast one launch sequence per mesh, with the
    single-mesh entry points (scratch preallocated, no graph)."""

    def __init__(self, batch: MeshBatch):
        self.b = batch
        L = _native.load()
        dev = batch.device
        self.trees = []
        self.meshes = []
        for m in range(batch.num_mesh):
            t0, t1 = int(batch.tri_off[m]), int(batch.tri_off[m + 1])
            v0, v1 = int(batch.vtx_off[m]), int(batch.vtx_off[m + 1])
            T = t1 - t0
            self.meshes.append((batch.tri2vtx[t0:t1], batch.vtx2xyz[v0:v1], T, v1 - v0))
            self.trees.append((torch.empty((2 * T - 1, 3), dtype=torch.uint32, device=dev),
                               torch.empty((2 * T - 1, 6), dtype=torch.float32, device=dev)))
        self.build_bytes = L.dm_trimesh3_build_scratch_bytes(batch.max_tri)
        self.build_scratch = torch.empty((self.build_bytes,), dtype=torch.uint8, device=dev)

    def build(self):
        sp = torch.cuda.current_stream(self.b.device).cuda_stream
        for (tri, vtx, T, V), (bvh, aabb) in zip(self.meshes, self.trees):
            _native.call("dm_trimesh3_make_bvhnodes_bvhnode2aabb", sp, T, tri.data_ptr(), V, vtx.data_ptr(),
                         bvh.data_ptr(), aabb.data_ptr(), self.build_scratch.data_ptr(), self.build_bytes)

    def alloc_cast(self, img_w: int, img_h: int):
        self.img_w, self.img_h = img_w, img_h
        n = img_w * img_h
        self.pix2tri = torch.empty((self.b.num_mesh, img_h, img_w), dtype=torch.uint32, device=self.b.device)
        self.pix2t = torch.empty((self.b.num_mesh, img_h, img_w), dtype=torch.float32, device=self.b.device)
        self.cast_bytes = _native.load().dm_cast_scratch_bytes(n, self.b.max_tri)
        self.cast_scratch = torch.empty((self.cast_bytes,), dtype=torch.uint8, device=self.b.device)

    def cast_pixels(self, transforms_colmajor: torch.Tensor):
        sp = torch.cuda.current_stream(self.b.device).cuda_stream
        for m, ((tri, vtx, T, V), (bvh, aabb)) in enumerate(zip(self.meshes, self.trees)):
            _native.call("dm_pix2tri_by_raycast", sp, self.img_w, self.img_h, self.pix2tri[m].data_ptr(),
                         self.pix2t[m].data_ptr(), T, tri.data_ptr(), V, vtx.data_ptr(), bvh.data_ptr(),
                         aabb.data_ptr(), transforms_colmajor[m].data_ptr(), self.cast_scratch.data_ptr(),
                         self.cast_bytes)
        return self.pix2tri, self.pix2t


def ortho_transforms(batch_meshes, margin: float = 0.05) -> np.ndarray:
    """(num_mesh, 16) column-major orthographic cameras looking down -z over
    each mesh's bounding box."""
    from .workloads import box_ortho_ndc2world
    return np.stack([box_ortho_ndc2world(v.min(0), v.max(0), margin) for _, v in batch_meshes]).astype(np.float32)
