"""Generates the golden fixtures under tests/golden/.

* ``ref_morton.npz`` / ``ref_topology.npz`` / ``ref_centroid.npz`` come from
  the reference's OWN code: del-msh-cuda-kernels/cuda/mortons.h and
  bvhnodes_morton.cu compiled as host C++ by oracle/build.py into oracle/_ref
  (needs the reference checkout; run in the container that has it).
* ``oracle_icosphere1280_256.npz`` is the oracle's result for the 1280-triangle jittered
  icosphere (build + 256x256 orthographic cast), stored with its inputs so the
  same bits can be checked on any machine.
* ``ref_assets.npz`` holds the reference's example meshes (asset/bunny_1k.obj,
  asset/spot/spot_triangulated.obj) read from the checkout, as inputs.

Usage: python tests/golden/make_golden.py <reference checkout> [assets]
"""
from __future__ import annotations

import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "del-msh_gb300"))

from oracle import build as obuild  # noqa: E402
from oracle import oracle as O  # noqa: E402
from del_msh_gb300 import workloads as W  # noqa: E402


def sorted_case(codes):
    codes = np.asarray(codes, np.uint32)
    idx = np.argsort(codes, kind="stable").astype(np.uint32)
    return idx, codes[idx]


def topology_cases():
    rng = np.random.default_rng(1234)
    cases = {}
    pts = rng.random((100, 3)).astype(np.float32)  # test_mortons.py:36-61 uses 100 random points
    cases["rand100"] = O.vtx2morton(pts, np.eye(4, dtype=np.float32).reshape(-1))
    cases["rand5000"] = rng.integers(0, 1 << 30, 5000, dtype=np.uint64).astype(np.uint32)
    cases["dup_small"] = rng.integers(0, 8, 3000, dtype=np.uint64).astype(np.uint32)
    cases["dup_runs"] = np.repeat(rng.integers(0, 1 << 30, 200, dtype=np.uint64), rng.integers(1, 40, 200)).astype(
        np.uint32)
    cases["all_equal"] = np.full(50, 12345, np.uint32)
    cases["n2"] = np.array([7, 3], np.uint32)
    cases["n2_equal"] = np.array([5, 5], np.uint32)
    cases["n3"] = np.array([9, 1, 4], np.uint32)
    cases["n3_equal"] = np.array([2, 2, 2], np.uint32)
    tri, vtx = W.clustered_soup(20000, seed=7)
    c = O.tri2cntr(tri, vtx)
    cases["soup20k"] = O.vtx2morton(c, O.fit_into_unit_preserve_asp(O.aabb3(c)))
    return cases


def load_obj_triangles(path):
    """Vertices and triangles of a Wavefront OBJ file of triangles (v x y z;
    f a[/t[/n]] b c with 1-based indices)."""
    vtx, tri = [], []
    for line in pathlib.Path(path).read_text().splitlines():
        f = line.split()
        if not f:
            continue
        if f[0] == "v":
            vtx.append([float(x) for x in f[1:4]])
        elif f[0] == "f":
            idx = [int(w.split("/")[0]) - 1 for w in f[1:]]
            if len(idx) != 3:
                raise ValueError(f"{path}: a face that is not a triangle")
            tri.append(idx)
    return np.array(tri, np.uint32), np.array(vtx, np.float32)


def write_assets(ref_root):
    """ref_assets.npz: the reference's two example meshes (asset/bunny_1k.obj,
    asset/spot/spot_triangulated.obj) as arrays, parity inputs of the GPU
    build and cast tests."""
    root = pathlib.Path(ref_root)
    out = {}
    for name, rel in (("bunny", "asset/bunny_1k.obj"), ("spot", "asset/spot/spot_triangulated.obj")):
        tri, vtx = load_obj_triangles(root / rel)
        out[f"{name}__tri2vtx"] = tri
        out[f"{name}__vtx2xyz"] = vtx
    np.savez_compressed(HERE / "ref_assets.npz", **out)


def main():
    obuild.build_oracle()
    ref = sys.argv[1] if len(sys.argv) > 1 else None
    if len(sys.argv) > 2 and sys.argv[2] == "assets":
        write_assets(obuild.reference_root(ref))
        return
    # the reference checkout: first argument, else DELMSH_REFERENCE
    if obuild.build_ref(ref) is None:
        raise SystemExit("usage: make_golden.py <reference checkout> (or set DELMSH_REFERENCE): the reference's "
                         "sources are required to regenerate the reference-code fixtures")
    R = O.ref_lib()
    rng = np.random.default_rng(99)

    # Morton codes of the reference's device_morton_code3 / device_expand_bits3
    pts = rng.uniform(-0.25, 1.25, (4000, 3)).astype(np.float32)
    special = np.array([[0, 0, 0], [1, 1, 1], [0, 0, 1], [1, 0, 1], [0.5, 0.5, 0.5], [1023 / 1024, 1, 0],
                        [-1e-7, 1 + 1e-7, 0.999999], [np.nan, 0.3, np.inf], [-np.inf, 0.7, 0.0009765625]],
                       np.float32)
    pts = np.concatenate([special, pts])
    codes = np.array([R.ref_morton_code3(float(x), float(y), float(z)) for x, y, z in pts], np.uint32)
    bits = np.array([R.ref_expand_bits3(i) for i in range(1024)], np.uint32)
    np.savez_compressed(HERE / "ref_morton.npz", pts=pts, codes=codes, expand_bits3=bits)

    # Radix-tree topology of the reference's kernel_MortonCode_BVHTopology
    out = {}
    for name, codes in topology_cases().items():
        idx, srt = sorted_case(codes)
        out[f"{name}__idx2obj"] = idx
        out[f"{name}__idx2morton"] = srt
        out[f"{name}__bvhnodes"] = O.ref_bvh_topology(srt, idx)
    np.savez_compressed(HERE / "ref_topology.npz", **out)

    # Triangle centroids of the reference's tri2cntr kernel
    tri, vtx = W.jittered_icosphere(2, seed=5)
    np.savez_compressed(HERE / "ref_centroid.npz", tri2vtx=tri, vtx2xyz=vtx, tri2cntr=O.ref_tri2cntr(tri, vtx))

    # Oracle snapshot of the 1280-triangle icosphere: build + 256^2 cast
    tri, vtx = W.jittered_icosphere(3, seed=0)
    r = O.build(tri, vtx)
    m = W.ortho_ndc2world()
    p2t, p2tt = O.pix2tri(tri, vtx, r["bvhnodes"], r["bvhnode2aabb"], m, 256, 256)
    np.savez_compressed(HERE / "oracle_icosphere1280_256.npz", tri2vtx=tri, vtx2xyz=vtx, transform=r["transform"],
                        tri2morton=r["tri2morton"], idx2tri=r["idx2tri"], idx2morton=r["idx2morton"],
                        bvhnodes=r["bvhnodes"], bvhnode2aabb=r["bvhnode2aabb"], ndc2world=m, pix2tri=p2t,
                        pix2t=p2tt)
    write_assets(obuild.reference_root(ref))
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main()
