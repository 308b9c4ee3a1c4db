"""The oracle's restatement of the reference's median-split ray order
(RaySort::operator(), src/core/RaySort.cpp:7-118, after RayBoundingbox), which
the coherence comparison (oracle/coherence.py) sets against the project's key."""
import numpy as np


def _axis(lo, hi):
    # RaySort.cpp:13-14: the index of the wider of x and y, then 2 if that
    # index is below the z extent (the reference compares the index itself)
    t = 1 if (hi[0] - lo[0]) < (hi[1] - lo[1]) else 0
    return 2 if t < (hi[2] - lo[2]) else t


def _rays(n, scale, seed):
    rng = np.random.default_rng(seed)
    org = (rng.uniform(-1, 1, (n, 3)) * np.asarray(scale)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return org, d


def test_median_split_order_is_a_permutation_split_at_the_median(built):
    _, oracle = built
    for scale, seed in (((10, 2, 0.5), 1), ((0.5, 3, 0.2), 2), ((1, 1, 4), 3)):
        org, d = _rays(20000, scale, seed)
        o = oracle.median_split_order(org, d)
        assert np.array_equal(np.sort(o), np.arange(20000))
        a = _axis(org.min(axis=0), org.max(axis=0))
        first, second = org[o[:10000], a], org[o[10000:], a]
        assert first.max() <= second.min()
        # quarters: each half is split again on its own box
        q = org[o[:5000]], org[o[5000:10000]]
        lo, hi = org.min(axis=0), org.max(axis=0)
        hi2 = hi.copy()
        hi2[a] = first.max()
        a2 = _axis(lo, hi2)
        assert q[0][:, a2].max() <= q[1][:, a2].min()


def test_small_ranges_keep_their_order_and_mid_ranges_sort_by_direction(built):
    _, oracle = built
    org, d = _rays(64, (1, 1, 1), 4)
    assert np.array_equal(oracle.median_split_order(org, d), np.arange(64))
    org, d = _rays(1000, (1, 1, 1), 5)
    o = oracle.median_split_order(org, d)
    # 65..4096 rays: sorted by direction along the axis chosen from the (origin) box
    a = _axis(org.min(axis=0), org.max(axis=0))
    assert d[o[:500], a].max() <= d[o[500:], a].min()
