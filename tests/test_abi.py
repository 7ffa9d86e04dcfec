"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/*.h (no GPU needed: nothing is called)."""
import ctypes
import pathlib
import re

ROOT = pathlib.Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(dm_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "dm_trimesh3_make_bvhnodes_bvhnode2aabb" in names
    assert "dm_pix2tri_by_raycast" in names
    assert len(names) >= 14


def test_library_exports_every_declared_symbol():
    from del_msh_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(str(path))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from del_msh_gb300 import _native
    assert set(declared_functions()) <= set(_native.exported_symbols())


def test_scratch_queries_without_gpu():
    from del_msh_gb300 import _native
    L = _native.load(build_if_missing=True)
    assert L.dm_trimesh3_build_scratch_bytes(2_097_152) > 16 * 2_097_152
    assert L.dm_cast_scratch_bytes(2_073_600, 2_097_152) >= 16 * 2_097_152
    assert L.dm_array1d_argsort_scratch_bytes(1000) > 8000
    assert L.dm_version().decode().startswith("delmsh_gb300")
