"""numpy <-> torch helpers for the tests (uint32 goes through an int32 view)."""
import numpy as np


def to_dev(a, torch, device="cuda:0"):
    a = np.ascontiguousarray(a)
    if a.dtype == np.uint32:
        return torch.from_numpy(a.view(np.int32)).to(device).view(torch.uint32)
    return torch.from_numpy(a).to(device)


def to_np(t, torch):
    if t.dtype == torch.uint32:
        return t.view(torch.int32).cpu().numpy().view(np.uint32)
    return t.cpu().numpy()


def bits(a):
    """Raw bits for exact comparison; every NaN is mapped to one pattern (NaN
    payloads differ between x86, Arm and CUDA and carry no information here)."""
    a = np.array(a, copy=True)
    if a.dtype == np.float32:
        a[np.isnan(a)] = np.float32("nan")
    return np.ascontiguousarray(a).view(np.uint32)


_CUBE_VTX = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])
_CUBE_TRI = np.array([[0, 2, 1], [0, 3, 2], [4, 5, 6], [4, 6, 7], [0, 1, 5], [0, 5, 4], [1, 2, 6], [1, 6, 5],
                      [2, 3, 7], [2, 7, 6], [3, 0, 4], [3, 4, 7]])


def voxel_cubes(rng, grid, num_cube, scale):
    """Surfaces of `num_cube` unit cubes at random cells of a grid^3 lattice,
    scaled by `scale` in f32 (so that lattice coordinates round), each face as
    two triangles whose vertex order is rotated at random.  Cubes may coincide
    or touch, so faces overlap and many hits lie on bounding-box faces."""
    cells = rng.integers(0, grid, size=(num_cube, 3))
    vtx = ((cells[:, None, :] + _CUBE_VTX[None]).reshape(-1, 3).astype(np.float32) * np.float32(scale))
    rot = rng.integers(0, 3, size=(num_cube, 12))
    cols = (np.arange(3)[None, None, :] + rot[:, :, None]) % 3
    tri = np.take_along_axis(np.broadcast_to(_CUBE_TRI, (num_cube, 12, 3)), cols, axis=2)
    tri = tri + 8 * np.arange(num_cube)[:, None, None]
    return np.ascontiguousarray(tri.reshape(-1, 3).astype(np.uint32)), np.ascontiguousarray(vtx)


def lattice_rays(rng, grid, scale, num_ray):
    """Rays from random points around the lattice aimed at lattice points or
    quarter points on its edges; about one coordinate in seven of the origin
    equals the target's, giving axis-parallel directions."""
    g = rng.integers(0, grid + 1, size=(num_ray, 3)).astype(np.float64)
    g += np.where(rng.random((num_ray, 3)) < 0.5, rng.integers(0, 4, size=(num_ray, 3)) * 0.25, 0.0)
    tgt = (g * scale).astype(np.float32)
    org = ((rng.random((num_ray, 3)) * 2 - 0.5) * (grid + 2) * scale).astype(np.float32)
    org = np.where(rng.random((num_ray, 3)) < 0.15, tgt, org)
    return np.ascontiguousarray(org), np.ascontiguousarray(tgt - org)


def reference_pin_torus():
    """The scene of del-msh-cpu's pix2tri test (pix2tri.rs:121-173): torus_zup
    (1.3, 0.4, 64, 32) in f32, rotated by 1.15 rad about x, then translated
    by (0.01, 0.61, 0.03); transform_ndc2world is the inverse of
    diag(0.5, 0.5, 0.5, 1), i.e. diag(2, 2, 2, 1) (column-major).  Returns
    (tri2vtx, vtx2xyz, ndc2world)."""
    import math
    from del_msh_gb300 import workloads as W
    f = np.float32
    nlg, nlt, R, r = 64, 32, f(1.3), f(0.4)
    rlg, rlt = f(2 * math.pi) / f(nlg), f(2 * math.pi) / f(nlt)
    ilg, ilt = np.meshgrid(np.arange(nlg, dtype=f), np.arange(nlt, dtype=f), indexing="ij")
    lg, lt = ilg * rlg, ilt * rlt
    r0 = R + r * np.cos(lt)
    vtx = np.stack([r0 * np.sin(lg), r0 * np.cos(lg), r * np.sin(lt)], -1).reshape(-1, 3).astype(f)
    c, s = f(math.cos(1.15)), f(math.sin(1.15))
    m = np.array([[1, 0, 0, 0.01], [0, c, -s, 0.61], [0, s, c, 0.03], [0, 0, 0, 1]], f)  # translate . rot_x
    vtx = ((vtx @ m[:3, :3].T) + m[:3, 3]).astype(f)
    ndc2world = np.array([2, 0, 0, 0, 0, 2, 0, 0, 0, 0, 2, 0, 0, 0, 0, 1], f)
    return W.torus_zup_topology(nlg, nlt), vtx, ndc2world
