"""The oracle's 26/98 direction bins against a plain restatement (CPU only).

Bins are the surface cells of an m^3 cube over [-1,1]^3 (m = 3 for 26, 5
for 98): a direction is scaled so that its largest component has magnitude 1,
each component falls into one of m equal intervals, and the cells are counted
in x-major order with the interior cells skipped."""
import math

import numpy as np
import pytest


def _bin(d, nbins):
    m = 3 if nbins == 26 else 5
    mx = max(abs(float(x)) for x in d)
    if not mx > 0:
        return 0
    inv = np.float32(1.0) / np.float32(mx)
    half = np.float32(0.5) * np.float32(m)
    c = [min(m - 1, max(0, int(math.floor(float((np.float32(x) * inv + np.float32(1.0)) * half))))) for x in d]
    surface = [(i, j, k) for i in range(m) for j in range(m) for k in range(m)
               if min(i, j, k) == 0 or max(i, j, k) == m - 1]
    return surface.index(tuple(c))


@pytest.mark.parametrize("nbins", [26, 98])
def test_oracle_bins_match_a_plain_restatement(built, nbins):
    _, oracle = built
    rng = np.random.default_rng(nbins)
    d = rng.normal(size=(3000, 3)).astype(np.float32)
    d[:8] = [[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, 0, -1], [1, 1, 1], [-1, -1, -1], [1, -1, 0.5], [0, 0, 0]]
    got = oracle.ray_bins(d, nbins)
    want = np.array([_bin(x, nbins) for x in d], np.int32)
    assert np.array_equal(got, want)
    assert len(np.unique(got)) == nbins


def test_oracle_six_bins_are_the_cardinal_bins(built):
    _, oracle = built
    d = np.random.default_rng(6).normal(size=(1000, 3)).astype(np.float32)
    assert np.array_equal(oracle.ray_bins(d, 6), oracle.cardinal(d))
