"""The grouped pool sweep (su2gpu_pool_set_sweep_groups): the chains split
into groups whose sweeps (one launch per pass, a graph per group) run on
several streams in turn, so that passes of different groups share the GPU.

* Same fields and counters as one launch per pass on one stream and as the
  persistent sweep, bit for bit: every kernel is the same, and a chain's
  passes keep their order on its group's stream; FP64 and FP32, graph and
  direct launches, several sweeps per call.
* The launch count, the setting and its precedence (a forced persistent mode
  wins; multicanonical chains turn it off), and the autotuner's choice, which
  leaves the chains untouched and gives the same results whatever it picks.
"""
import numpy as np
import pytest

from native import hot_fields
from su2higgs_gb300 import abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from su2higgs_gb300 import gpu as g
    g.lib()
    return g


def as_dict(f):
    return {n: getattr(f, n) for n in ("link", "u1", "d0", "d1", "trip", "sing")}


def specs_of(content, precision, n=9):
    sides = [(8, 8, 8), (12, 6, 10), (4, 4, 4), (16, 16, 16), (24, 20, 22), (10, 10, 10), (6, 8, 4), (14, 12, 16),
             (8, 12, 6), (20, 16, 18), (12, 12, 12), (16, 8, 12)]
    return [(abi.make_params(content, L=sides[k % len(sides)], betasu2=6.0 + k, msq_triplet=-0.2 + 0.05 * k,
                             precision=precision), 300 + k, k) for k in range(n)]


def make_pool(gpu, specs, inputs, mode):
    pool = gpu.Pool(specs[0][0], arena_bytes=256 << 20, max_chains=16)
    slots = []
    for (p, seed, chain), f in zip(specs, inputs):
        s = pool.add(p, seed=seed, chain=chain)
        pool.upload(s, **f)
        slots.append(s)
    if mode == "persistent":
        pool.persistent = True
    elif mode == "per_pass":
        pool.persistent = False
    else:
        pool.sweep_groups = mode
    return pool, slots


def assert_same(pa, sa, pb, sb):
    for x, y in zip(sa, sb):
        fa, fb = pa.download(x), pb.download(y)
        for n in fa:
            if fa[n] is not None:
                assert np.array_equal(fa[n], fb[n]), (x, n, float(np.abs(fa[n] - fb[n]).max()))
        assert np.array_equal(pa.counters(x), pb.counters(y)), x


@pytest.mark.parametrize("content,precision", [("fund", 64), ("adj", 64), ("su2u1s", 64), ("higgs2", 64),
                                               ("fund", 32), ("adj", 32), ("su2u1s", 32)])
@pytest.mark.parametrize("graph", [True, False])
def test_grouped_equals_other_modes(gpu, content, precision, graph):
    specs = specs_of(content, precision)
    inputs = [as_dict(hot_fields(p, seed=400 + k, phi_mean=0.5)) for k, (p, _, _) in enumerate(specs)]
    pools = [make_pool(gpu, specs, inputs, m) for m in ("per_pass", (4, 3), (9, 2), "persistent")]
    # groups balance sites, so uneven chains can give fewer groups than asked
    g1, g2 = pools[1][0].sweep_groups, pools[2][0].sweep_groups
    assert 2 <= g1[0] <= 4 and g1[1] == 3 and 2 <= g2[0] <= 9 and g2[1] == 2
    assert pools[0][0].sweep_groups == (0, 1) and pools[3][0].sweep_groups == (0, 1)
    for n in (1, 3, 2):
        for pool, _ in pools:
            pool.run(n, graph=graph)
    for pool, slots in pools[1:]:
        assert_same(pools[0][0], pools[0][1], pool, slots)
    ms = [pool.measure() for pool, _ in pools]
    for m in ms[1:]:
        assert sorted(m) == sorted(ms[0])
        for k in m:
            assert np.array_equal(ms[0][k], m[k]), k
    for pool, _ in pools:
        pool.close()


def test_grouped_launch_count_and_precedence(gpu):
    specs = specs_of("adj", 32)
    inputs = [as_dict(hot_fields(p, seed=k)) for k, (p, _, _) in enumerate(specs)]
    pool, slots = make_pool(gpu, specs, inputs, "per_pass")
    per_sweep = pool.launches_per_sweep()
    assert per_sweep == 6 + 10 + 1
    pool.persistent = None
    pool.sweep_groups = (3, 2)
    g, ns = pool.sweep_groups
    assert 2 <= g <= 3 and ns == 2 and not pool.persistent
    assert pool.launches_per_sweep() == g * per_sweep
    # a forced persistent mode wins over the groups
    pool.persistent = True
    assert pool.sweep_groups == (0, 1) and pool.persistent
    pool.persistent = None
    assert pool.sweep_groups == (g, 2)
    # more groups than chains: at most one chain each
    pool.sweep_groups = (50, 4)
    g50, ns = pool.sweep_groups
    assert g <= g50 <= len(specs) and ns == 4
    pool.sweep_groups = None
    assert pool.sweep_groups == (0, 1)
    with pytest.raises(gpu.SU2GPUError):
        pool.sweep_groups = (4, 0)
    # a multicanonical chain turns the groups off
    pool.sweep_groups = (3, 2)
    from native import WeightBuf
    f = pool.download(slots[0])
    w = WeightBuf(16, orderparam=abi.SIGMASQ, mode=abi.MUCA_READONLY)
    sig = float(np.sum(0.5 * np.sum(f["trip"] ** 2, axis=1)) / specs[0][0].sites())
    w.pos[1:] = np.linspace(sig - 1, sig + 1, 17)
    w.pos[0] = sig - 1000
    w.linearize()
    s = w.struct
    s.min, s.max, s.wrk_min, s.wrk_max = sig - 1, sig + 1, sig - 1, sig + 1
    pool.muca_set(slots[0], s)
    assert pool.sweep_groups == (0, 1)
    pool.run(1)
    pool.close()


def test_autotuner_grouped_choice_keeps_results(gpu):
    """The autotuner may pick the grouped mode (timed on a scratch copy: the
    chains do not advance); whatever it picks, the chains then follow the
    same trajectories as in a pool swept one launch per pass."""
    specs = specs_of("adj", 32, n=12)
    inputs = [as_dict(hot_fields(p, seed=500 + k)) for k, (p, _, _) in enumerate(specs)]
    a, sa = make_pool(gpu, specs, inputs, "per_pass")
    b, sb = make_pool(gpu, specs, inputs, None)
    b.persistent = None
    c0 = [b.counters(s).copy() for s in sb]
    b.autotune()
    for s, c in zip(sb, c0):
        assert np.array_equal(b.counters(s), c)
    g, n = b.sweep_groups
    assert g == 0 or (2 <= g <= len(specs) and 1 <= n <= 8)
    for k in (2, 3):
        a.run(k)
        b.run(k)
    assert_same(a, sa, b, sb)
    a.close()
    b.close()
