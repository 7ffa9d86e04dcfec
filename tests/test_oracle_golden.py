"""The oracle (CPU restatement of del-msh-cpu) against the reference's own
known answers and against golden vectors produced by the reference's code."""
import numpy as np


def test_expand_bits3_known_answers(oracle):
    # del-msh-cpu/src/mortons.rs:83-87
    L = oracle.lib()
    assert L.or_expand_bits3(0b11111111) == 0b001001001001001001001001
    assert L.or_expand_bits3(0b10001001) == 0b001000000000001000000001


def test_morton_code3_known_answers(oracle):
    # del-msh-cpu/src/mortons.rs:104-110
    L = oracle.lib()
    assert L.or_morton_code3(0.0, 0.0, 0.0) == 0
    assert L.or_morton_code3(0.0, 0.0, 1.0) == 0b001001001001001001001001001001
    assert L.or_morton_code3(1.0, 0.0, 1.0) == 0b101101101101101101101101101101
    assert L.or_morton_code3(1.0, 1.0, 1.0) == 0xFFFFFFFF >> 2


def test_morton_code2_known_answers(oracle):
    # del-msh-cpu/src/mortons.rs:29-33
    L = oracle.lib()
    assert L.or_morton_code2(0.0, 0.0) == 0
    assert L.or_morton_code2(0.0, 1.0) == 0b01010101010101010101010101010101


def test_morton_matches_reference_code(oracle, golden_dir):
    g = np.load(golden_dir / "ref_morton.npz")
    L = oracle.lib()
    got = np.array([L.or_morton_code3(float(x), float(y), float(z)) for x, y, z in g["pts"]], np.uint32)
    assert np.array_equal(got, g["codes"])
    assert np.array_equal(np.array([L.or_expand_bits3(i) for i in range(1024)], np.uint32), g["expand_bits3"])


def test_centroids_match_reference_code(oracle, golden_dir):
    g = np.load(golden_dir / "ref_centroid.npz")
    got = oracle.tri2cntr(g["tri2vtx"], g["vtx2xyz"])
    assert np.array_equal(got.view(np.uint32), g["tri2cntr"].view(np.uint32))


def test_topology_matches_reference_code(oracle, golden_dir):
    g = np.load(golden_dir / "ref_topology.npz")
    names = sorted({k.split("__")[0] for k in g.files})
    assert len(names) >= 10
    for name in names:
        idx, srt, ref = g[f"{name}__idx2obj"], g[f"{name}__idx2morton"], g[f"{name}__bvhnodes"]
        got = oracle.update_bvhnodes(idx, srt)
        assert np.array_equal(got, ref), name
        assert oracle.check_bvh_topology(got, idx.size), name
        assert oracle.check_morton_code_range_split(srt), name


def test_stable_argsort_ties_by_index(oracle):
    codes = np.array([5, 3, 5, 1, 3, 5, 0], np.uint32)
    idx, srt = oracle.argsort_stable(codes)
    assert idx.tolist() == [6, 3, 1, 4, 0, 2, 5]
    assert srt.tolist() == sorted(codes.tolist())


def test_oracle_snapshot_icosphere1280(oracle, golden_dir):
    """The committed oracle result of the 1280-triangle icosphere reproduces
    bit for bit on this machine (x86 and Arm alike)."""
    g = np.load(golden_dir / "oracle_icosphere1280_256.npz")
    r = oracle.build(g["tri2vtx"], g["vtx2xyz"])
    for k in ("transform", "tri2morton", "idx2tri", "idx2morton", "bvhnodes", "bvhnode2aabb"):
        assert np.array_equal(np.asarray(r[k]).view(np.uint32), g[k].view(np.uint32)), k
    p2t, p2tt = oracle.pix2tri(g["tri2vtx"], g["vtx2xyz"], r["bvhnodes"], r["bvhnode2aabb"], g["ndc2world"], 256, 256,
                               threads=4)
    assert np.array_equal(p2t, g["pix2tri"])
    assert np.array_equal(p2tt.view(np.uint32), g["pix2t"].view(np.uint32))
