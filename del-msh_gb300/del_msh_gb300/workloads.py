"""Seeded synthetic meshes, cameras and rays for the LBVH build / ray-cast path.

Every generator is deterministic for a given seed (numpy PCG64).  Vertices are
built in float64 and rounded once to float32; indices are uint32.  Geometry
formulas that need sin/cos can differ in the last float64 bit between libm
builds, so fixtures that must be reproducible across machines store the
generated arrays rather than the seed.

Matrices are returned as float32 arrays of 16 entries in column-major order
(the layout del-msh's kernels read, ``Mortons/torch.py:42``).
"""
from __future__ import annotations

import math

import numpy as np

UMAX = 0xFFFFFFFF


# ------------------------------------------------------------------ meshes

def icosphere(level: int, radius: float = 1.0):
    """Icosahedron subdivided ``level`` times by edge midpoints projected onto
    the sphere: V = 10*4^level + 2, T = 20*4^level."""
    g = (1.0 + math.sqrt(5.0)) / 2.0
    v = [(-1, g, 0), (1, g, 0), (-1, -g, 0), (1, -g, 0), (0, -1, g), (0, 1, g), (0, -1, -g), (0, 1, -g),
         (g, 0, -1), (g, 0, 1), (-g, 0, -1), (-g, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    vtx = np.array(v, np.float64)
    vtx /= np.linalg.norm(vtx, axis=1, keepdims=True)
    tri = np.array(f, np.int64)
    for _ in range(level):
        e = np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]])
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        mid = vtx[uniq[:, 0]] + vtx[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = vtx.shape[0]
        vtx = np.concatenate([vtx, mid])
        nt = tri.shape[0]
        m01, m12, m20 = inv[:nt] + base, inv[nt:2 * nt] + base, inv[2 * nt:] + base
        a, b, c = tri[:, 0], tri[:, 1], tri[:, 2]
        tri = np.concatenate([np.stack([a, m01, m20], 1), np.stack([b, m12, m01], 1), np.stack([c, m20, m12], 1),
                              np.stack([m01, m12, m20], 1)])
    return tri.astype(np.uint32), (vtx * radius).astype(np.float32)


def _icosahedron():
    """The 20 faces (outward winding) and 12 unit corners of ``icosphere(0)``."""
    tri, _ = icosphere(0)
    g = (1.0 + math.sqrt(5.0)) / 2.0
    c = np.array([(-1, g, 0), (1, g, 0), (-1, -g, 0), (1, -g, 0), (0, -1, g), (0, 1, g), (0, -1, -g),
                  (0, 1, -g), (g, 0, -1), (g, 0, 1), (-g, 0, -1), (-g, 0, 1)], np.float64)
    return tri.astype(np.int64), c / np.linalg.norm(c, axis=1, keepdims=True)


def geodesic_sphere(freq: int, radius: float = 1.0):
    """Icosphere of any subdivision frequency: every icosahedron face is cut
    into freq^2 triangles on its barycentric grid and the grid points are
    projected onto the sphere, so V = 10*freq^2 + 2 and T = 20*freq^2 (freq =
    2^level has the counts of ``icosphere(level)``).  A point shared by faces
    is keyed by its (corner, weight) pairs in ascending corner order and its
    position is summed in that order, so every face computes it identically."""
    freq = int(freq)
    if freq < 1 or freq > 4095:
        raise ValueError("freq must be in 1..4095")
    faces, corners = _icosahedron()
    n = freq
    r, c = np.tril_indices(n + 1)  # grid point (row r, column c <= r), index r(r+1)/2 + c
    w = np.stack([n - r, r - c, c], axis=1)  # weights on the face's corners a, b, c
    ids = np.repeat(faces[:, None, :], r.size, axis=1)  # [face, point, 3]
    ww = np.broadcast_to(w[None], ids.shape).copy()
    ids = np.where(ww > 0, ids, 15)  # a zero weight drops its corner from the key
    order = np.argsort(ids, axis=2, kind="stable")
    ids = np.take_along_axis(ids, order, 2)
    ww = np.take_along_axis(ww, order, 2)
    key = ((ids[..., 0] << 56) | (ww[..., 0] << 40) | (ids[..., 1] << 36) | (ww[..., 1] << 20) |
           (ids[..., 2] << 16) | ww[..., 2])
    uniq, first, inv = np.unique(key.reshape(-1), return_index=True, return_inverse=True)
    fi, ii = ids.reshape(-1, 3)[first], ww.reshape(-1, 3)[first]
    pos = np.zeros((uniq.size, 3))
    cext = np.concatenate([corners, np.zeros((4, 3))])  # id 15 (no corner) adds +0
    for k in range(3):
        pos = pos + cext[fi[:, k]] * (ii[:, k:k + 1] / n)
    pos /= np.linalg.norm(pos, axis=1, keepdims=True)
    vid = inv.reshape(faces.shape[0], r.size)

    def at(rr, cc):
        return (rr * (rr + 1)) // 2 + cc

    up_r, up_c = np.tril_indices(n)  # (r, c) with c <= r < n
    up = np.stack([at(up_r, up_c), at(up_r + 1, up_c), at(up_r + 1, up_c + 1)], 1)
    dn_r, dn_c = np.tril_indices(n, -1)  # (r, c) with c < r < n
    dn = np.stack([at(dn_r, dn_c), at(dn_r + 1, dn_c + 1), at(dn_r, dn_c + 1)], 1)
    local = np.concatenate([up, dn])
    tri = vid[:, local].reshape(-1, 3)
    return tri.astype(np.uint32), (pos * radius).astype(np.float32)


def jittered_icosphere(level: int = 3, radius: float = 1.0, jitter: float = 0.01, seed: int = 0):
    """Icosphere with every vertex coordinate moved by seeded U(-jitter, jitter)."""
    tri, vtx = icosphere(level, radius)
    rng = np.random.default_rng(seed)
    vtx = (vtx.astype(np.float64) + rng.uniform(-jitter, jitter, vtx.shape)).astype(np.float32)
    return tri, vtx


def torus_zup_topology(ndiv_major: int, ndiv_minor: int):
    """Triangle list of del-msh-cpu ``trimesh3_primitive::torus_zup``
    (trimesh3_primitive.rs:326-371): two triangles per grid quad, vertex
    ``ilg*ndiv_minor + ilt``."""
    ilg, ilt = np.meshgrid(np.arange(ndiv_major), np.arange(ndiv_minor), indexing="ij")
    iug = (ilg + 1) % ndiv_major
    iut = (ilt + 1) % ndiv_minor
    v00 = ilg * ndiv_minor + ilt
    v11 = iug * ndiv_minor + iut
    v10 = iug * ndiv_minor + ilt
    v01 = ilg * ndiv_minor + iut
    t = np.stack([v00, v11, v10, v00, v01, v11], axis=-1).reshape(-1, 3)
    return t.astype(np.uint32)


def torus_zup(major_radius: float, minor_radius: float, ndiv_major: int, ndiv_minor: int, disp=None):
    """Vertices of ``torus_zup`` (trimesh3_primitive.rs:326-371) with an
    optional radial displacement ``disp[ilg, ilt]`` along the tube normal."""
    lg = np.arange(ndiv_major, dtype=np.float64)[:, None] * (2 * math.pi / ndiv_major)
    lt = np.arange(ndiv_minor, dtype=np.float64)[None, :] * (2 * math.pi / ndiv_minor)
    r = minor_radius + (0.0 if disp is None else disp)
    r0 = major_radius + r * np.cos(lt)
    xyz = np.stack(np.broadcast_arrays(r0 * np.sin(lg), r0 * np.cos(lg), r * np.sin(lt)), axis=-1)
    return torus_zup_topology(ndiv_major, ndiv_minor), xyz.reshape(-1, 3).astype(np.float32)


def displaced_torus(ndiv: int = 1024, major_radius: float = 1.0, minor_radius: float = 0.3, amplitude: float = 0.02,
                    num_freq: int = 8, seed: int = 0):
    """Torus on an ndiv x ndiv grid (2*ndiv^2 triangles) displaced along the
    tube normal by a seeded sum of ``num_freq`` sinusoids with integer
    frequencies in 1..64, scaled so the peak amplitude is ``amplitude``."""
    rng = np.random.default_rng(seed)
    fa = rng.integers(1, 65, num_freq)
    fb = rng.integers(1, 65, num_freq)
    ph = rng.uniform(0, 2 * math.pi, num_freq)
    w = rng.uniform(0.5, 1.0, num_freq)
    lg = np.arange(ndiv, dtype=np.float64)[:, None] * (2 * math.pi / ndiv)
    lt = np.arange(ndiv, dtype=np.float64)[None, :] * (2 * math.pi / ndiv)
    d = np.zeros((ndiv, ndiv))
    for k in range(num_freq):
        d += w[k] * np.sin(fa[k] * lg + fb[k] * lt + ph[k])
    d *= amplitude / w.sum()
    return torus_zup(major_radius, minor_radius, ndiv, ndiv, disp=d)


def clustered_soup(num_tri: int = 4_194_304, num_cluster: int = 32, sigma: float = 1e-3, half: float = 5e-4,
                   seed: int = 0):
    """Triangle soup whose centroids come from ``num_cluster`` Gaussian
    clusters (std ``sigma``, clipped to the unit cube); each vertex is the
    centroid plus U(-half, half)^3.  V = 3T, tri i = (3i, 3i+1, 3i+2)."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.0, 1.0, (num_cluster, 3))
    which = rng.integers(0, num_cluster, num_tri)
    cog = np.clip(centres[which] + rng.normal(0.0, sigma, (num_tri, 3)), 0.0, 1.0)
    vtx = cog[:, None, :] + rng.uniform(-half, half, (num_tri, 3, 3))
    tri = np.arange(3 * num_tri, dtype=np.uint32).reshape(-1, 3)
    return tri, vtx.reshape(-1, 3).astype(np.float32)


# ----------------------------------------------------------------- cameras

def ortho_ndc2world(half_width: float = 1.2, z_near: float = 2.0, z_far: float = -2.0) -> np.ndarray:
    """Orthographic ndc->world map: ndc (x, y, +1) -> (hw*x, hw*y, z_near) and
    (x, y, -1) -> (hw*x, hw*y, z_far); rays run along -z when z_near > z_far."""
    m = np.eye(4)
    m[0, 0] = m[1, 1] = half_width
    m[2, 2] = (z_near - z_far) / 2.0
    m[2, 3] = (z_near + z_far) / 2.0
    return colmajor(m)


def box_ortho_ndc2world(lo, hi, margin: float = 0.05) -> np.ndarray:
    """Orthographic camera looking down -z over the xy extent of a box."""
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    c = (lo + hi) / 2
    h = (hi - lo) / 2 * (1 + margin) + 1e-6
    m = np.eye(4)
    m[0, 0], m[0, 3] = h[0], c[0]
    m[1, 1], m[1, 3] = h[1], c[1]
    z_near, z_far = hi[2] + h[2] + 0.1, lo[2] - h[2] - 0.1
    m[2, 2] = (z_near - z_far) / 2.0
    m[2, 3] = (z_near + z_far) / 2.0
    return colmajor(m)


def look_at(eye, target, up):
    eye, target, up = (np.asarray(a, np.float64) for a in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    if np.linalg.norm(s) < 1e-9:
        s = np.cross(f, np.array([1.0, 0.0, 0.0]))
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    v = np.eye(4)
    v[0, :3], v[1, :3], v[2, :3] = s, u, -f
    v[:3, 3] = -v[:3, :3] @ eye
    return v


def perspective(fovy_deg: float, aspect: float, near: float, far: float):
    """Projection with ndc z = +1 on the near plane and -1 on the far plane, so
    that del-msh's pixel ray (origin at ndc z=+1, towards z=-1) points away
    from the eye (the Blender-style convention of Mat44/torch.py:143-206)."""
    fy = 1.0 / math.tan(math.radians(fovy_deg) / 2)
    p = np.zeros((4, 4))
    p[0, 0] = fy / aspect
    p[1, 1] = fy
    p[2, 2] = (near + far) / (far - near)
    p[2, 3] = 2 * near * far / (far - near)
    p[3, 2] = -1.0
    return p


def pinhole_ndc2world(eye, target=(0, 0, 0), up=(0, 0, 1), fovy_deg=60.0, aspect=16 / 9, near=0.05, far=10.0):
    w2n = perspective(fovy_deg, aspect, near, far) @ look_at(eye, target, up)
    return colmajor(np.linalg.inv(w2n))


def random_viewpoint(radius: float = 3.0, seed: int = 0):
    rng = np.random.default_rng(seed)
    d = rng.normal(size=3)
    return d / np.linalg.norm(d) * radius


def colmajor(m: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(m, np.float64).T.reshape(-1)).astype(np.float32)


# -------------------------------------------------------------------- rays

def cube_boundary_rays(num_ray: int, seed: int = 0, lo: float = 0.0, hi: float = 1.0):
    """Origins uniform on the faces of [lo,hi]^3, directions uniform over the
    inward hemisphere of the face."""
    rng = np.random.default_rng(seed)
    face = rng.integers(0, 6, num_ray)
    axis, side = face // 2, face % 2
    org = rng.uniform(lo, hi, (num_ray, 3))
    org[np.arange(num_ray), axis] = np.where(side == 0, lo, hi)
    d = rng.normal(size=(num_ray, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    inward = np.where(side == 0, 1.0, -1.0)
    flip = d[np.arange(num_ray), axis] * inward < 0
    d[flip] *= -1
    return org.astype(np.float32), d.astype(np.float32)


# ------------------------------------------------------- ragged mesh batches

def ragged_batch(num_mesh: int = 4096, tmin: int = 64, tmax: int = 65536, jitter: float = 0.01, seed: int = 0):
    """``num_mesh`` seeded jittered icospheres / tori with triangle counts
    log-uniform in [tmin, tmax].  Returns a list of (tri2vtx, vtx2xyz).

    Each drawn target t is realised as closely as the mesh family allows,
    never above tmax: an icosphere of frequency f = round(sqrt(t/20)) (20 f^2
    triangles, ``geodesic_sphere``), or a torus grid of n_minor =
    round(sqrt(t/4)) by n_major = round(t / (2 n_minor)) quads (2 n_major
    n_minor triangles).  Over [64, 65536] the batch averages about 9.4k
    triangles per mesh, 38.7M for 4096 meshes."""
    rng = np.random.default_rng(seed)
    target = np.exp(rng.uniform(math.log(tmin), math.log(tmax), num_mesh))
    kinds = rng.integers(0, 2, num_mesh)
    ico_cache = {}
    meshes = []
    fmax = max(1, int(math.floor(math.sqrt(tmax / 20.0))))
    for i in range(num_mesh):
        t = float(target[i])
        if kinds[i] == 0:
            f = int(np.clip(round(math.sqrt(t / 20.0)), 1, fmax))
            if f not in ico_cache:
                ico_cache[f] = geodesic_sphere(f)
            tri, vtx = ico_cache[f]
        else:
            nminor = max(3, int(round(math.sqrt(t / 4.0))))
            nmajor = max(3, int(round(t / (2.0 * nminor))))
            while 2 * nmajor * nminor > tmax and nmajor > 3:
                nmajor -= 1
            tri, vtx = torus_zup(1.0, 0.35, nmajor, nminor)
        vtx = (vtx.astype(np.float64) + rng.uniform(-jitter, jitter, vtx.shape)).astype(np.float32)
        meshes.append((tri, vtx))
    return meshes
