"""Traversal work of the 1920x1080 pinhole cast of the displaced 2,097,152-
triangle torus, counted by the oracle's recursion on one CPU thread.

TEST INFRASTRUCTURE ONLY: a measurement aid, never on the product path.

The GPU cast makes the recursion's decisions (search_bvh3.rs:103-221), so the
counts are its work too.  Each branch entered reads its node record and tests
its two children's boxes; each triangle test reads the leaf's record, the
triangle's three indices and three vertices.  Traversal bytes per ray, the
figure set against L2 bandwidth:

    (2 * branches + 1) * 36 B  (12 B node record + 24 B box, root included)
  + tri_tests * 48 B           (12 B indices + 36 B vertices)

    python -m oracle.traversal_work [--cast-ms MS]

With ``--cast-ms`` (a measured cast time) it also prints the bandwidth those
bytes imply.
"""
from __future__ import annotations

import argparse
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "del-msh_gb300"))

from del_msh_gb300 import workloads as W  # noqa: E402

from . import oracle as O  # noqa: E402

IMG_W, IMG_H, NDIV, SEED = 1920, 1080, 1024, 0


def traversal_bytes(work):
    return (2 * work["branches"] + work["rays"]) * 36 + work["tri_tests"] * 48


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--cast-ms", type=float, default=None, help="measured GPU cast time of one image")
    a = ap.parse_args(argv)
    tri, vtx = W.displaced_torus(NDIV, seed=SEED)
    m = W.pinhole_ndc2world(W.random_viewpoint(3.0, seed=SEED), aspect=IMG_W / IMG_H)
    r = O.build(tri, vtx)
    work = O.pix2tri_work(tri, vtx, r["bvhnodes"], r["bvhnode2aabb"], m, IMG_W, IMG_H)
    b = traversal_bytes(work)
    out = dict(work, branches_per_ray=work["branches"] / work["rays"], tri_tests_per_ray=work["tri_tests"] / work["rays"],
               traversal_bytes=b, traversal_bytes_per_ray=b / work["rays"])
    if a.cast_ms:
        out["cast_ms"] = a.cast_ms
        out["traversal_gbs"] = b / (a.cast_ms * 1e-3) / 1e9
    print(json.dumps(out))


if __name__ == "__main__":
    main()
