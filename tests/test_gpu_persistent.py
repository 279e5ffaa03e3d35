"""The persistent pool sweep (k_pool_persist): one launch works through the
(sweep, pass, tile) list of every chain, each tile waiting only for its own
chain's previous pass.

* Same results as one launch per pass, bit for bit: fields and counters of
  every chain, FP64 and FP32, graph and direct launches, several sweeps per
  launch, chains of uneven sizes, a single chain (every pass then waits for
  the previous one), and the pipelined cycle.  The per-site code is the same
  source in both modes and the random numbers are keyed by chain, site, sweep
  and pass, not by block or order of execution.
* The bounded dependency wait: a work list whose dependencies never finish
  makes every wait give up; the kernel ends, reports flag 4, and leaves the
  fields and sweep counters untouched; the pool works normally afterwards.
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


def specs_of(content, precision):
    base = dict(precision=precision)
    return [
        (abi.make_params(content, L=(8, 8, 8), betasu2=6.0, **base), 11, 0),
        (abi.make_params(content, L=(12, 6, 10), betasu2=9.5, msq_triplet=-0.2, msq_phi=-0.05, **base), 12, 1),
        (abi.make_params(content, L=(4, 4, 4), betasu2=12.0, **base), 11, 2),
        (abi.make_params(content, L=(16, 16, 16), **base), 13, 3),
        (abi.make_params(content, L=(24, 20, 22), betasu2=7.0, **base), 14, 4),
    ]


def make_pool(gpu, specs, persistent, inputs):
    pool = gpu.Pool(specs[0][0], arena_bytes=128 << 20, max_chains=8)
    pool.persistent = persistent
    slots = []
    for (p, seed, chain), f in zip(specs, inputs):
        s = pool.add(p, seed=seed, chain=chain)
        pool.upload(s, **f)
        slots.append(s)
    return pool, slots


def assert_same(pa, sa, pb, sb):
    for x, y in zip(sa, sb):
        fa, fb = pa.download(x), pb.download(y)
        for n in fa:
            if fa[n] is not None:
                d = np.abs(fa[n] - fb[n])
                assert np.array_equal(fa[n], fb[n]), (x, n, float(d.max()), int(np.count_nonzero(d)))
        assert np.array_equal(pa.counters(x), pb.counters(y)), x


@pytest.mark.parametrize("content,precision", [("fund", 64), ("adj", 64), ("su2u1s", 64), ("higgs2", 64),
                                               ("fundadj", 64), ("fund", 32), ("adj", 32), ("su2u1s", 32)])
@pytest.mark.parametrize("graph", [True, False])
def test_persistent_equals_per_pass(gpu, content, precision, graph):
    specs = specs_of(content, precision)
    inputs = [as_dict(hot_fields(p, seed=200 + k, phi_mean=0.5)) for k, (p, _, _) in enumerate(specs)]
    a, sa = make_pool(gpu, specs, True, inputs)
    b, sb = make_pool(gpu, specs, False, inputs)
    assert a.persistent and not b.persistent
    for n in (1, 3, 2):
        a.run(n, graph=graph)
        b.run(n, graph=graph)
    assert_same(a, sa, b, sb)
    ma, mb = a.measure(), b.measure()
    for x, y in zip(sa, sb):
        assert np.array_equal(ma[x], mb[y])


@pytest.mark.parametrize("precision", [64, 32])
def test_persistent_single_chain(gpu, precision):
    p = abi.make_params("adj", L=(32, 32, 32), precision=precision)
    f = [as_dict(hot_fields(p, seed=5, phi_mean=0.5))]
    a, sa = make_pool(gpu, [(p, 3, 0)], True, f)
    b, sb = make_pool(gpu, [(p, 3, 0)], False, f)
    a.run(4)
    b.run(4)
    assert_same(a, sa, b, sb)


def test_persistent_cycle_equals_per_pass(gpu):
    specs = specs_of("su2u1s", 32)
    inputs = [as_dict(hot_fields(p, seed=300 + k, phi_mean=0.5)) for k, (p, _, _) in enumerate(specs)]
    outs = []
    for persistent in (True, False):
        pool, slots = make_pool(gpu, specs, persistent, inputs)
        fields = [{n: v.copy() for n, v in f.items() if v is not None} for f in inputs]
        sums = pool.cycle(slots, fields, 3)
        outs.append((fields, sums, [pool.counters(s) for s in slots]))
    (fa, ma, ca), (fb, mb, cb) = outs
    for x, y in zip(fa, fb):
        for n in x:
            assert np.array_equal(x[n], y[n]), n
    assert np.array_equal(ma, mb)
    for x, y in zip(ca, cb):
        assert np.array_equal(x, y)


def test_persistent_wait_gives_up(gpu):
    specs = specs_of("adj", 32)[:3]
    inputs = [as_dict(hot_fields(p, seed=400 + k, phi_mean=0.5)) for k, (p, _, _) in enumerate(specs)]
    pool, slots = make_pool(gpu, specs, True, inputs)
    ref, rslots = make_pool(gpu, specs, True, inputs)
    before = [pool.download(s) for s in slots]
    flags = pool.check_wait_timeout(spin_limit=500)
    assert flags & 4, flags
    for s, f in zip(slots, before):
        got = pool.download(s)
        for n in f:
            if f[n] is not None:
                assert np.array_equal(got[n], f[n]), n
    # the flags were cleared and the sweep counters did not move: the pool
    # goes on exactly as one that never ran the check
    pool.run(2)
    ref.run(2)
    assert_same(pool, slots, ref, rslots)


def test_persistent_launch_count(gpu):
    specs = specs_of("adj", 32)[:2]
    inputs = [as_dict(hot_fields(p, seed=1)) for p, _, _ in specs]
    pool, _ = make_pool(gpu, specs, True, inputs)
    assert pool.launches_per_sweep() == 2
    pool.persistent = False
    assert pool.launches_per_sweep() == 6 + 10 + 1


def test_persistent_automatic_mode(gpu):
    """Automatic (default) mode: persistent for 8 chains or more with enough
    tiles per pass (16 per resident block), one launch per pass otherwise."""
    p = abi.make_params("adj", L=(8, 8, 8), precision=32)
    pool = gpu.Pool(p, arena_bytes=64 << 20, max_chains=16)
    slots = []
    for k in range(8):
        slots.append(pool.add(p, seed=k, chain=k))
        pool.upload(slots[-1], **as_dict(hot_fields(p, seed=k)))
    assert not pool.persistent  # 16 tiles per pass
    pool.persistent = True
    assert pool.persistent
    pool.persistent = None
    assert not pool.persistent
    pool.close()
    from su2higgs_gb300 import workloads
    specs = workloads.batched_ensemble(384)
    need = sum(gpu.Pool.chain_bytes(q) for q, _, _ in specs)
    big = gpu.Pool(specs[0][0], arena_bytes=need, max_chains=384)
    for q, seed, chain in specs:
        big.add(q, seed=seed, chain=chain)
    assert big.persistent  # the 384-chain ensemble: 43k tiles per pass
    big.close()


def test_autotuner_picks_the_persistent_item_size(gpu):
    """On the 384-chain ensemble the autotuner times the persistent sweep's
    work-item sizes on a scratch copy (the chains do not advance) and keeps
    one of them; sweeps with the pick equal one-launch-per-pass sweeps."""
    from su2higgs_gb300 import workloads
    specs = workloads.batched_ensemble(384)
    need = sum(gpu.Pool.chain_bytes(q) for q, _, _ in specs)
    pools = []
    for persistent in (None, False):
        pool = gpu.Pool(specs[0][0], arena_bytes=need, max_chains=384)
        for q, seed, chain in specs:
            s = pool.add(q, seed=seed, chain=chain)
            if chain % 97 == 0:
                pool.upload(s, **workloads.hot_fields(q, seed))
        pool.persistent = persistent
        pools.append(pool)
    a, b = pools
    assert a.persistent and not b.persistent
    before = a.download(0)
    a.autotune()
    assert a.persist_tiles in (4, 6, 8, 12, 16, 24, 32)
    for n in before:
        if before[n] is not None:
            assert np.array_equal(a.download(0)[n], before[n]), n
    a.run(2)
    b.run(2)
    for s in (0, 97, 194, 291):
        fa, fb = a.download(s), b.download(s)
        for n in fa:
            if fa[n] is not None:
                assert np.array_equal(fa[n], fb[n]), (s, n)
        assert np.array_equal(a.counters(s), b.counters(s)), s


def test_error_flags_reported_once(gpu):
    """A kernel error flag (set here from the host, as a kernel that found a
    bad state would) makes the next run fail with ERR_KERNEL and is cleared
    by it: the run after that works."""
    specs = specs_of("adj", 32)[:3]
    inputs = [as_dict(hot_fields(p, seed=410 + k)) for k, (p, _, _) in enumerate(specs)]
    pool, slots = make_pool(gpu, specs, True, inputs)
    pool.raise_error(4)
    with pytest.raises(gpu.SU2GPUError, match="flags 4"):
        pool.run(1)
    pool.run(2)
    m = pool.measure()
    assert all(np.all(np.isfinite(v)) for v in m.values())


def test_long_recipe_sweeps_one_launch_per_pass(gpu):
    """A recipe of more passes than the persistent work list holds (6 link
    + 2 x 41 triplet passes = 88 > 64): forcing the persistent mode is
    refused, the automatic mode sweeps one launch per pass, and the
    pipelined cycle gives the same fields as upload + run + download."""
    specs = [(abi.make_params("adj", L=(8, 8, 8), precision=32, scalar_sweeps=40, betasu2=6.0 + k), 20 + k, k)
             for k in range(8)]
    inputs = [as_dict(hot_fields(p, seed=430 + k)) for k, (p, _, _) in enumerate(specs)]
    pool, slots = make_pool(gpu, specs, None, inputs)
    with pytest.raises(gpu.SU2GPUError, match="passes per sweep"):
        pool.persistent = True
    assert not pool.persistent
    assert pool.launches_per_sweep() == 6 + 82 + 1
    fields = [{n: v.copy() for n, v in f.items() if v is not None} for f in inputs]
    sums = pool.cycle(slots, fields, 2)
    ref, rslots = make_pool(gpu, specs, False, inputs)
    ref.run(2)
    for s, f in zip(rslots, fields):
        got = ref.download(s)
        for n in f:
            assert np.array_equal(got[n], f[n]), n
    mref = ref.measure()
    assert np.array_equal(np.array([mref[s] for s in rslots]), sums)


@pytest.mark.parametrize("precision", [32, 64])
def test_persistent_shapes_bit_identical(gpu, precision):
    """Both launch shapes of the persistent sweep give the fields of one
    launch per pass bit for bit."""
    specs = specs_of("adj", precision)
    inputs = [as_dict(hot_fields(p, seed=500 + k, phi_mean=0.5)) for k, (p, _, _) in enumerate(specs)]
    ref, rslots = make_pool(gpu, specs, False, inputs)
    ref.run(3)
    for shape in (0, 1):
        pool, slots = make_pool(gpu, specs, True, inputs)
        pool.persist_shape = shape
        assert pool.persist_shape[0] == shape and pool.persist_shape[1] == 128
        pool.run(3)
        assert_same(pool, slots, ref, rslots)
