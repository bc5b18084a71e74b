"""Order and counting rules of the hierarchy (hrchy_space.cc:36-231)."""
from math import comb

import numpy as np
import pytest

import oracle


@pytest.mark.parametrize("K,N", [(1, 4), (2, 5), (3, 10), (5, 3), (4, 6), (14, 4), (9, 2)])
def test_count_order_and_links(K, N):
    n, p1, m1 = oracle.Oracle("port").hrchy(K, N)
    count = n.shape[0]
    assert count == comb(K + N, N)
    tiers = n.sum(axis=1)
    assert np.all(np.diff(tiers) >= 0)              # tier ascending
    for t in range(N + 1):                          # descending lexicographic within a tier
        block = [tuple(r) for r in n[tiers == t]]
        assert block == sorted(block, reverse=True)
    void = count
    for l in range(count):
        for k in range(K):
            up = n[l].copy(); up[k] += 1
            dn = n[l].copy(); dn[k] -= 1
            if tiers[l] < N:
                assert np.array_equal(n[p1[l, k]], up)
            else:
                assert p1[l, k] == void
            if n[l, k] > 0:
                assert np.array_equal(n[m1[l, k]], dn)
            else:
                assert m1[l, k] == void
    assert np.all(p1[void] == void) and np.all(m1[void] == void)
