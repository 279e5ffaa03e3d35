"""The pass order of the random_sweeps mode (update.c:278-300, 338-344 of
su2higgs): the library's host-side order (su2gpu_sweep_order) equals the
oracle's, every link repetition is a shuffle of the reference's parity and
direction arrays, and the orders are uniformly distributed (the reference's
Fisher-Yates shuffle, update.c:461-468, on an unbiased 64-bit stream).  No
GPU is needed: the order is computed on the host."""
import collections

import numpy as np
import pytest
from scipy import stats

from native import oracle_sweep_order


@pytest.fixture(scope="module")
def gpu():
    from su2higgs_gb300 import build
    build.build()
    from su2higgs_gb300 import gpu as g
    return g


@pytest.mark.parametrize("update_links,scalar_sweeps", [(1, 4), (3, 0), (0, 2), (2, 7)])
def test_library_order_equals_oracle(gpu, update_links, scalar_sweeps):
    for seed, chain, sweep in [(1, 0, 0), (314, 2, 41), (2 ** 62 + 5, 0x40000000, 99999), (7, 11, 2 ** 31)]:
        d, q, f = gpu.sweep_order(seed, chain, sweep, update_links, scalar_sweeps)
        od, oq, of = oracle_sweep_order(seed, chain, sweep, update_links, scalar_sweeps)
        assert np.array_equal(d, od) and np.array_equal(q, oq) and np.array_equal(f, of)
        for k in range(update_links):
            assert sorted(d[k]) == [0, 0, 1, 1, 2, 2]
            assert sorted(q[k]) == [0, 0, 0, 1, 1, 1]
        assert set(f) <= {0, 1}


def test_orders_differ_between_sweeps_and_chains(gpu):
    a = gpu.sweep_order(5, 0, 10)
    b = gpu.sweep_order(5, 0, 11)
    c = gpu.sweep_order(5, 1, 10)
    assert any(not np.array_equal(x, y) for x, y in zip(a, b))
    assert any(not np.array_equal(x, y) for x, y in zip(a, c))
    again = gpu.sweep_order(5, 0, 10)
    assert all(np.array_equal(x, y) for x, y in zip(a, again))


def test_order_distribution_is_uniform(gpu):
    """Over many sweeps: the 20 distinct parity patterns and the 90 direction
    patterns of 6 entries come up equally often (chi^2), the first pass's
    parity and direction independently of each other, and the scalar first
    parity is EVEN half of the time."""
    n = 20000
    par, dirs, pair, first = collections.Counter(), collections.Counter(), collections.Counter(), 0
    for s in range(n):
        d, q, f = gpu.sweep_order(20261203, 3, s, 1, 0)
        par[tuple(q[0])] += 1
        dirs[tuple(d[0])] += 1
        pair[(tuple(q[0])[0], tuple(d[0])[0])] += 1
        first += int(f[0] == 0)
    assert len(par) == 20 and len(dirs) == 90  # C(6,3) parity patterns, 6!/(2!)^3 direction patterns
    for cnt in (par, dirs, pair):
        obs = np.array(list(cnt.values()), float)
        p = stats.chisquare(obs).pvalue
        assert p > 1e-4, p
    z = (first - n / 2) / np.sqrt(n / 4)
    assert abs(z) < 4.5, z
