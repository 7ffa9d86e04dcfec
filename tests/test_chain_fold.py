"""The warp tier's chain fold, checked on the CPU.

The cast's warp tier (csrc/dm_traverse.cuh) evaluates a run of chain links
(branch j with leaf j as left child and branch j + 1 as right child) as a
fold from the run's far end, instead of walking the links.  This file
restates, in float32 numpy, the traversal's recursive result F(node) (the
rules of search_bvh3.rs:103-221 as the kernels implement them) and the fold.
It checks the fold against the plain recursion, and both against the
oracle's cast, on a duplicate-heavy soup whose runs of equal Morton codes
build long chains.
"""
import sys

import numpy as np

from del_msh_gb300 import workloads as W

F32 = np.float32
NONE_ID = 0xFFFFFFFF
NONE = (F32(np.inf), NONE_ID)
FOLD_MIN = 8  # the kernels' kFoldMin


def pick(a, b):
    """Keep b (the later result) unless a is strictly closer; none is the identity."""
    if a[1] == NONE_ID:
        return b
    if b[1] == NONE_ID:
        return a
    return a if a[0] < b[0] else b


class Caster:
    def __init__(self, tri, vtx, bvh, aabb, org, d):
        self.tri, self.vtx, self.bvh, self.aabb = tri, vtx, bvh.astype(np.int64), aabb
        self.org = org.astype(np.float32)
        self.d = d.astype(np.float32)
        with np.errstate(divide="ignore"):
            self.inv = (F32(1) / self.d).astype(np.float32)
        self.T = tri.shape[0]

    def slab(self, n):
        box = self.aabb[n]
        tmin, tmax = F32(-np.inf), F32(np.inf)
        for a in range(3):
            lo, hi, o, inv, dd = box[a], box[3 + a], self.org[a], self.inv[a], self.d[a]
            if dd != 0:
                t0 = F32(F32(lo - o) * inv)
                t1 = F32(F32(hi - o) * inv)
                tmin = np.fmax(tmin, np.fmin(t0, t1))
                tmax = np.fmin(tmax, np.fmax(t0, t1))
            elif o < lo or o > hi:
                return None
        if not (tmin <= tmax) or tmax < 0:
            return None
        return (tmin, tmax)

    def leaf_hit(self, leaf):
        it = int(self.bvh[leaf][1])
        p0, p1, p2 = (self.vtx[int(v)] for v in self.tri[it])

        def cross(a, b):
            return np.array([F32(a[1] * b[2]) - F32(a[2] * b[1]), F32(a[2] * b[0]) - F32(a[0] * b[2]),
                             F32(a[0] * b[1]) - F32(a[1] * b[0])], np.float32)

        def dot(a, b):
            return F32(F32(F32(a[0] * b[0]) + F32(a[1] * b[1])) + F32(a[2] * b[2]))

        e1, e2, tv = (p1 - p0).astype(np.float32), (p2 - p0).astype(np.float32), (self.org - p0).astype(np.float32)
        pv = cross(self.d, e2)
        det = dot(e1, pv)
        if det == 0:
            return NONE
        inv_det = F32(F32(1) / det)
        u = F32(dot(tv, pv) * inv_det)
        if not (u >= 0 and u <= 1):
            return NONE
        qv = cross(tv, e1)
        v = F32(dot(self.d, qv) * inv_det)
        if not (v >= 0 and F32(u + v) <= 1):
            return NONE
        t = F32(dot(e2, qv) * inv_det)
        if not (t >= 0) or not (t < np.inf):
            return NONE
        return (t, it)

    @staticmethod
    def tuple_lt(a, b):
        return a[1] < b[1] if a[0] == b[0] else a[0] < b[0]

    def is_link(self, n):
        return n < self.T - 1 and self.bvh[n][1] == self.T - 1 + n and self.bvh[n][2] == n + 1

    def branch(self, n, f):
        """F(n) for a branch, the children searched with f."""
        left, right = int(self.bvh[n][1]), int(self.bvh[n][2])
        hl, hr = self.slab(left), self.slab(right)
        if hl is None and hr is None:
            return NONE
        near_left = self.tuple_lt(hl, hr) if (hl is not None and hr is not None) else hl is not None
        near, far = (left, right) if near_left else (right, left)
        r1 = f(near)
        if hl is None or hr is None:
            return r1
        far_enter = hr[0] if near_left else hl[0]
        if r1[1] != NONE_ID and far_enter > r1[0]:
            return r1
        return pick(r1, f(far))

    def F(self, n):
        if self.bvh[n][2] == NONE_ID:
            return self.leaf_hit(n)
        return self.branch(n, self.F)

    def F_fold(self, n):
        if self.bvh[n][2] == NONE_ID:
            return self.leaf_hit(n)
        if self.is_link(n):
            c1 = n
            while self.is_link(c1 + 1):
                c1 += 1
            if c1 - n + 1 >= FOLD_MIN:
                tail = c1 + 1
                x = self.F_fold(tail) if self.slab(tail) is not None else NONE
                for j in range(c1, n - 1, -1):
                    leaf = self.T - 1 + j
                    ha, hb = self.slab(leaf), self.slab(j + 1)
                    h = self.leaf_hit(leaf) if ha is not None else NONE
                    if ha is None and hb is None:
                        x = NONE
                    elif hb is None:
                        x = h
                    elif ha is not None:
                        if self.tuple_lt(ha, hb):
                            x = h if (h[1] != NONE_ID and hb[0] > h[0]) else pick(h, x)
                        else:
                            x = x if (x[1] != NONE_ID and ha[0] > x[0]) else pick(x, h)
                return x
        return self.branch(n, self.F_fold)

    def cast(self, fold):
        if self.slab(0) is None:
            return NONE
        return self.F_fold(0) if fold else self.F(0)


def test_chain_fold_equals_recursion_and_oracle(oracle):
    sys.setrecursionlimit(100000)
    tri, vtx = W.clustered_soup(6_000, num_cluster=2, seed=4)
    ref = oracle.build(tri, vtx)
    bvh, aabb = ref["bvhnodes"], ref["bvhnode2aabb"]
    T = tri.shape[0]
    links = sum(1 for n in range(T - 1) if bvh[n][1] == T - 1 + n and bvh[n][2] == n + 1)
    assert links > T // 4  # the soup's runs of equal codes build long chains
    org, _ = W.cube_boundary_rays(64, seed=4)
    rng = np.random.default_rng(4)
    target = vtx[tri[rng.integers(0, T, org.shape[0])]].mean(axis=1)
    d = (target + rng.uniform(-2e-4, 2e-4, target.shape) - org).astype(np.float32)
    r_hit, r_t = oracle.cast_rays(org, d, tri, vtx, bvh, aabb)
    hits = 0
    for k in range(org.shape[0]):
        c = Caster(tri, vtx, bvh, aabb, org[k], d[k])
        a, b = c.cast(False), c.cast(True)
        assert a[1] == b[1] and np.float32(a[0]).view(np.uint32) == np.float32(b[0]).view(np.uint32), k
        assert a[1] == r_hit[k], (k, a, r_hit[k])
        if a[1] != NONE_ID:
            assert np.float32(a[0]).view(np.uint32) == np.float32(r_t[k]).view(np.uint32), k
            hits += 1
    assert hits > org.shape[0] // 2


class CountingCaster(Caster):
    """The recursion with counters: branches entered and triangles tested."""

    def __init__(self, *a):
        super().__init__(*a)
        self.branches = 0
        self.tri_tests = 0

    def leaf_hit(self, leaf):
        self.tri_tests += 1
        return super().leaf_hit(leaf)

    def branch(self, n, f):
        self.branches += 1
        return super().branch(n, f)


def test_oracle_work_counts_match_recursion(oracle):
    """or_pix2tri_work's counts (the traversal-bytes figure) equal the
    restated recursion's, ray by ray summed over a small pinhole image."""
    tri, vtx = W.jittered_icosphere(3, seed=2)
    ref = oracle.build(tri, vtx)
    bvh, aabb = ref["bvhnodes"], ref["bvhnode2aabb"]
    m = W.pinhole_ndc2world(W.random_viewpoint(3.0, seed=2), aspect=1.0)
    w = h = 24
    work = oracle.pix2tri_work(tri, vtx, bvh, aabb, m, w, h)
    branches = tri_tests = hits = 0
    for i in range(w * h):
        org, d = oracle.ray_for_pixel(i, w, h, m)
        c = CountingCaster(tri, vtx, bvh, aabb, org, d)
        hits += c.cast(False)[1] != NONE_ID
        branches += c.branches
        tri_tests += c.tri_tests
    assert work == {"rays": w * h, "branches": branches, "tri_tests": tri_tests}
    assert hits > w * h // 4 and tri_tests >= hits
