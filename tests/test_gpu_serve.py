"""The request server: every result is the same alone, in a concurrent mix
and through the plain serial path (bit for bit), build+cast results equal the
oracle, and a small memory budget forces evictions without changing results."""
import numpy as np
import pytest

from helpers import bits

pytestmark = pytest.mark.gpu


def _workload():
    from del_msh_gb300.serve import ServedWorkload
    return ServedWorkload(num_mesh=6, tmin=500, tmax=30000, img=48, num_ray=1500, seed=7, ring=1)


def _requests(wl):
    """A fixed mix: builds, refits to frames 1..3 (some repeated), ray casts at
    several frames, each request with its own output buffer."""
    from del_msh_gb300.serve import BUILD_CAST, CAST_RAYS, REFIT_CAST
    spec = []
    for m in range(6):
        spec += [(BUILD_CAST, m, 0), (REFIT_CAST, m, 1), (CAST_RAYS, m, 1), (REFIT_CAST, m, 2), (CAST_RAYS, m, 0),
                 (REFIT_CAST, m, 3), (BUILD_CAST, m, 2), (CAST_RAYS, m, 3)]
    rng = np.random.default_rng(0)
    spec = [spec[i] for i in rng.permutation(len(spec))]
    outs = [np.zeros(wl.max_out, np.uint32) for _ in spec]
    reqs = [wl.request(k, m, f, out=o) for (k, m, f), o in zip(spec, outs)]
    return spec, reqs, outs


def _n(wl, kind):
    return wl.num_ray if kind == 2 else wl.img * wl.img


def test_served_alone_mix_plain_identical(cuda, oracle):
    from del_msh_gb300.serve import BUILD_CAST, Server
    wl = _workload()
    with Server(budget_bytes=4 << 30, num_slots=4, max_tri=wl.max_tri, max_out=wl.max_out) as srv:
        wl.register_all(srv)
        spec, reqs, mix_outs = _requests(wl)
        res = srv.run_trace(reqs, [0.0] * len(reqs))  # all at once: maximal overlap
        assert all(r.status == 0 for r in res)
        mix = [o[:_n(wl, k)].copy() for (k, _, _), o in zip(spec, mix_outs)]
        _, reqs2, alone_outs = _requests(wl)
        for r in reqs2:
            assert srv.submit_and_wait(r).status == 0
        alone = [o[:_n(wl, k)].copy() for (k, _, _), o in zip(spec, alone_outs)]
        _, reqs3, plain_outs = _requests(wl)
        res3 = srv.run_plain(reqs3, [0.0] * len(reqs3))
        assert all(r.status == 0 for r in res3)
        plain = [o[:_n(wl, k)].copy() for (k, _, _), o in zip(spec, plain_outs)]
        st = srv.stats()
    for i in range(len(spec)):
        assert np.array_equal(mix[i], alone[i]), spec[i]
        assert np.array_equal(mix[i], plain[i]), spec[i]
    assert st["refits"] > 0 and st["builds"] > 0 and st["resident_hits"] > 0
    # build+cast at the rest pose is the single-mesh result of the oracle
    for (k, m, f), out in zip(spec, mix):
        if k == BUILD_CAST and f == 0:
            t, v = wl.meshes[m]
            ref = oracle.build(t, v)
            r_p2t, _ = oracle.pix2tri(t, v, ref["bvhnodes"], ref["bvhnode2aabb"], wl.cams[m], wl.img, wl.img)
            assert np.array_equal(out, r_p2t.reshape(-1)), m
    from del_msh_gb300 import _native
    assert _native.device_status(clear=True) == 0


def test_small_budget_evicts_and_keeps_results(cuda):
    from del_msh_gb300.serve import Server
    wl = _workload()
    with Server(budget_bytes=4 << 30, num_slots=2, max_tri=wl.max_tri, max_out=wl.max_out) as big:
        wl.register_all(big)
        spec, reqs, outs_big = _requests(wl)
        big.run_trace(reqs, [0.0] * len(reqs))
        st = big.stats()
        slots = st["bytes_slots"]
        per_mesh = st["bytes_resident"] / max(1, st["meshes_resident"])
    budget = int(slots + 2.5 * per_mesh)  # room for about two meshes
    with Server(budget_bytes=budget, num_slots=2, max_tri=wl.max_tri, max_out=wl.max_out) as small:
        wl.register_all(small)
        _, reqs2, outs_small = _requests(wl)
        res = small.run_trace(reqs2, [0.0] * len(reqs2))
        st2 = small.stats()
    assert all(r.status == 0 for r in res)
    assert st2["evictions"] > 0
    assert st2["bytes_resident"] + st2["bytes_slots"] <= budget
    for (k, _, _), a, b in zip(spec, outs_big, outs_small):
        assert np.array_equal(a[:_n(wl, k)], b[:_n(wl, k)])
