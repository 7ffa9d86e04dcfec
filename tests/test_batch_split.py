"""The on-chip batched build shares a mesh of T triangles over a cluster of
kC blocks (2 or 4), block r holding positions r*per .. r*per+per-1 with
per = ceil(T / kC), and finds a position's block with a multiply-high by
magic = floor((2^32 - 1) / per) + 1 (SegSplit in csrc/batch.cu).  Clusters
build only meshes of 16385..65536 triangles (pairs of blocks only up to
32768), so per lies in 4097..16384 and positions below 65536; this checks the
quotient for every such pair, and for the pairs' share sizes up to 32768."""
import numpy as np


def test_multiply_high_owner_is_exact():
    i = np.arange(65536, dtype=np.uint64)
    for kc in (2, 4):
        pers = sorted({(t + kc - 1) // kc for t in range(16385, 65537)})
        assert pers[0] > 4096 and pers[-1] <= 32768
        for per in pers:
            magic = np.uint64(0xFFFFFFFF // per + 1)
            own = (i * magic) >> np.uint64(32)
            assert np.array_equal(own, i // np.uint64(per)), (kc, per)


def test_divider_multiply_high_is_exact():
    """The casts' per-ray index arithmetic (Divider in csrc/dm_device.cuh)
    divides a 32-bit index n by d as the high 64 bits of n * ceil(2^64 / d):
    the product exceeds n / d by less than n / 2^64 < 1 / d, so the floor is
    exact.  Checked here on the edges and on random operands."""
    rng = np.random.default_rng(7)
    ds = [2, 3, 5, 7, 16, 30, 60, 64, 120, 480, 481, 1919, 4096, 65535, 65537, 2**31 - 1, 2**32 - 1]
    ds += [int(x) for x in rng.integers(2, 2**32, 300)]
    for d in ds:
        magic = (2**64 - 1) // d + 1
        ns = [0, 1, d - 1, d, d + 1, 2**32 - 1, 2**32 - 2, (2**32 - 1) // d * d, (2**32 - 1) // d * d - 1]
        ns += [int(x) for x in rng.integers(0, 2**32, 200)]
        for n in ns:
            if 0 <= n < 2**32:
                assert (n * magic) >> 64 == n // d, (n, d)
