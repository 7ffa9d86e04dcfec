"""Build recipe for the oracle (test infrastructure, never the product).

* ``build_oracle()`` compiles ``oracle.c`` (the CPU restatement of
  del-msh-cpu's LBVH build and ray cast) into ``oracle/_build/liboracle.so``
  with ``-ffp-contract=off`` so f32 arithmetic rounds as Rust's does.
* ``build_ref(root)`` compiles the reference's own CUDA sources for the path
  (``del-msh-cuda-kernels/cuda/bvhnodes_morton.cu`` + ``mortons.h``) as host
  C++ through ``ref_shim.cpp`` into ``oracle/_ref/libref_topology.so``.  It
  needs the reference checkout, given as ``root`` or by the
  ``DELMSH_REFERENCE`` environment variable; without one (as on a machine that
  only runs the tests) it does nothing.
"""
from __future__ import annotations

import os
import pathlib
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
BUILD_DIR = HERE / "_build"
REF_DIR = HERE / "_ref"
LIB_ORACLE = BUILD_DIR / "liboracle.so"
LIB_REF = REF_DIR / "libref_topology.so"
COMMON_FLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]


def _stale(out: pathlib.Path, *srcs: pathlib.Path) -> bool:
    return not out.exists() or any(s.stat().st_mtime > out.stat().st_mtime for s in srcs)


def build_oracle(force: bool = False) -> pathlib.Path:
    BUILD_DIR.mkdir(exist_ok=True)
    src, hdr = HERE / "oracle.c", HERE / "oracle.h"
    if force or _stale(LIB_ORACLE, src, hdr):
        tmp = LIB_ORACLE.with_suffix(".so.tmp")
        subprocess.run(["gcc", "-std=c11", *COMMON_FLAGS, "-pthread", str(src), "-o", str(tmp), "-lm"],
                       check=True)
        os.replace(tmp, LIB_ORACLE)
    return LIB_ORACLE


def reference_root(root=None) -> pathlib.Path | None:
    root = root or os.environ.get("DELMSH_REFERENCE")
    return pathlib.Path(root) if root else None


def build_ref(root=None, force: bool = False) -> pathlib.Path | None:
    ref = reference_root(root)
    if ref is None:
        return None
    kdir = ref / "del-msh-cuda-kernels" / "cuda"
    if not (kdir / "bvhnodes_morton.cu").exists():
        return None
    REF_DIR.mkdir(exist_ok=True)
    shim = HERE / "ref_shim.cpp"
    if force or _stale(LIB_REF, shim, kdir / "bvhnodes_morton.cu", kdir / "mortons.h"):
        tmp = LIB_REF.with_suffix(".so.tmp")
        subprocess.run(["g++", "-std=c++17", *COMMON_FLAGS, "-x", "c++", "-I", str(kdir), str(shim),
                        "-o", str(tmp)], check=True)
        os.replace(tmp, LIB_REF)
    return LIB_REF


if __name__ == "__main__":
    import sys
    print(build_oracle(force=True))
    print(build_ref(sys.argv[1] if len(sys.argv) > 1 else None, force=True))
