"""Multicanonical chains in pools (su2gpu_pool_muca_set): a global accept /
reject after every checked half-sweep of each chain with a weight
(muca_check, update.c:13-30; multicanonical.c:385-445).

* FP64: a pool chain with a weight follows a single-lattice context with the
  same parameters, seed, chain id and weight: the same decisions (counters
  and multicanonical counters equal, hits equal), fields equal to rounding
  (1e-9 after three sweeps, as the other pool tests), the order parameter to
  1e-9 -- in the persistent sweep and with one launch per pass, READONLY and
  FAST (the weight recursion every 5 checks).
* Both sweep modes give the same fields, counters and weight state bit for
  bit (FP32 and FP64), with chains with and without weights mixed.
* The autotuner's scratch sweeps leave the weight state alone; batch uploads
  and unsupported settings are refused.
"""

import numpy as np
import pytest

from native import WeightBuf, hot_fields
from su2higgs_gb300 import abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from su2higgs_gb300 import gpu as g
    g.lib()
    return g


def as_dict(f):
    return {n: getattr(f, n) for n in ("link", "u1", "d0", "d1", "trip", "sing") if getattr(f, n) is not None}


def weight_around(op, center, mode=abi.MUCA_READONLY, bins=24, width=0.25, steep=300.0):
    """A piecewise-linear weight over [center - width, center + width]."""
    w = WeightBuf(bins, orderparam=op, mode=mode)
    lo, hi = center - width, center + width
    w.pos[1:] = np.linspace(lo, hi, bins + 1)
    w.pos[0] = lo - 1000 * (hi - lo)
    w.W[1:] = steep * (w.pos[1:] - center) ** 2
    w.W[0] = w.W[1]
    w.W[bins + 1] = w.W[bins]
    w.linearize()
    s = w.struct
    s.min, s.max, s.wrk_min, s.wrk_max = lo, hi, lo, hi
    s.delta = 0.5
    if mode == abi.MUCA_FAST:
        s.update_interval = 5
    return w


def order_parameter(f, op, V):
    if op == abi.SIGMASQ:
        return float(np.sum(0.5 * np.sum(f.trip ** 2, axis=1)) / V)
    return float(np.sum(0.5 * np.sum(f.d0 ** 2, axis=1)) / V)


CASES = [("fund", abi.PHISQ), ("su2u1s", abi.PHISQ), ("adj", abi.SIGMASQ)]


def specs_of(content, precision):
    base = dict(precision=precision)
    return [
        (abi.make_params(content, L=(8, 8, 8), betasu2=6.0, **base), 11, 0),
        (abi.make_params(content, L=(12, 6, 10), betasu2=9.5, msq_triplet=-0.2, msq_phi=-0.05, **base), 12, 1),
        (abi.make_params(content, L=(6, 6, 6), betasu2=12.0, **base), 13, 2),
    ]


def make_pool(gpu, specs, inputs, weights, persistent):
    pool = gpu.Pool(specs[0][0], arena_bytes=64 << 20, max_chains=8)
    pool.persistent = persistent
    slots = []
    for (p, seed, chain), f, w in zip(specs, inputs, weights):
        s = pool.add(p, seed=seed, chain=chain)
        pool.upload(s, **as_dict(f))
        if w is not None:
            pool.muca_set(s, w.struct)
        slots.append(s)
    return pool, slots


def weights_for(specs, inputs, op, mode):
    # chains 0 and 1 with a weight, chain 2 without
    out = []
    for k, ((p, _, _), f) in enumerate(zip(specs, inputs)):
        out.append(weight_around(op, order_parameter(f, op, p.sites()), mode) if k < 2 else None)
    return out


def state(pool, slot, bins):
    w = WeightBuf(bins)
    pool.muca_get(slot, w.struct)
    s = w.struct
    return dict(pv=(s.param_value[0], s.param_value[1]), hits=w.hits.copy(), W=w.W.copy(),
                count=s.muca_count, delta=s.delta)


@pytest.mark.parametrize("content,op", CASES)
@pytest.mark.parametrize("persistent", [True, False])
@pytest.mark.parametrize("mode", [abi.MUCA_READONLY, abi.MUCA_FAST])
def test_pool_muca_chain_follows_single_context(gpu, content, op, persistent, mode):
    specs = specs_of(content, 64)
    inputs = [hot_fields(p, seed=70 + k, phi_mean=0.6, trip_sigma=0.5) for k, (p, _, _) in enumerate(specs)]
    weights = weights_for(specs, inputs, op, mode)
    pool, slots = make_pool(gpu, specs, inputs, weights, persistent)
    pool.run(3)
    for k in range(2):
        p, seed, chain = specs[k]
        ws = weights_for(specs, inputs, op, mode)[k]
        lat = gpu.Lattice(p, seed=seed, chain=chain)
        lat.upload(**as_dict(inputs[k]))
        lat.muca_set(ws.struct)
        lat.calc_orderparam(0)
        lat.calc_orderparam(1)
        lat.run_sweeps(0, 3, graph=False)
        got, want = pool.download(slots[k]), lat.download()
        for n in got:
            if got[n] is not None:
                assert np.max(np.abs(got[n] - want[n])) < 1e-9, n
        assert np.array_equal(pool.counters(slots[k])[:22], lat.counters()[:22])
        assert pool.counters(slots[k])[abi.C_TOTAL_MUCA] == 3 * 10
        a = state(pool, slots[k], 24)
        wl = WeightBuf(24)
        lat.muca_get(wl.struct)
        assert np.allclose(a["pv"], (wl.struct.param_value[0], wl.struct.param_value[1]), rtol=1e-9, atol=0)
        assert np.array_equal(a["hits"], wl.hits)
        assert np.max(np.abs(a["W"] - wl.W)) < 1e-9
        assert a["count"] == wl.struct.muca_count
        lat.close()
    # the chain without a weight makes no check
    assert pool.counters(slots[2])[abi.C_TOTAL_MUCA] == 0
    pool.close()


@pytest.mark.parametrize("precision", [32, 64])
@pytest.mark.parametrize("content,op", CASES)
def test_pool_muca_modes_bit_identical(gpu, content, op, precision):
    specs = specs_of(content, precision)
    p64 = [abi.make_params(content, L=tuple(p.L[:3])) for p, _, _ in specs]
    inputs = [hot_fields(q, seed=80 + k, phi_mean=0.6, trip_sigma=0.5) for k, q in enumerate(p64)]
    out = []
    for persistent in (True, False):
        weights = weights_for(specs, inputs, op, abi.MUCA_FAST)
        pool, slots = make_pool(gpu, specs, inputs, weights, persistent)
        pool.run(4)
        out.append(([pool.download(s) for s in slots], [pool.counters(s) for s in slots],
                    [state(pool, s, 24) for s in slots[:2]]))
        pool.close()
    (fa, ca, sa), (fb, cb, sb) = out
    for x, y in zip(fa, fb):
        for n in x:
            if x[n] is not None:
                assert np.array_equal(x[n], y[n]), n
    for x, y in zip(ca, cb):
        assert np.array_equal(x, y)
    # some checks rejected, so the restores ran
    assert sum(int(c[abi.C_TOTAL_MUCA] - c[abi.C_ACC_MUCA]) for c in ca[:2]) > 0
    for x, y in zip(sa, sb):
        assert x["pv"] == y["pv"] and np.array_equal(x["hits"], y["hits"]) and np.array_equal(x["W"], y["W"])


def test_pool_muca_autotune_leaves_the_weight_alone(gpu):
    specs = specs_of("fund", 32)
    inputs = [hot_fields(abi.make_params("fund", L=tuple(p.L[:3])), seed=90 + k, phi_mean=0.6)
              for k, (p, _, _) in enumerate(specs)]
    weights = weights_for(specs, inputs, abi.PHISQ, abi.MUCA_FAST)
    pool, slots = make_pool(gpu, specs, inputs, weights, None)
    before = [state(pool, s, 24) for s in slots[:2]]
    c0 = [pool.counters(s).copy() for s in slots]
    pool.autotune()
    after = [state(pool, s, 24) for s in slots[:2]]
    for x, y in zip(before, after):
        assert x["pv"] == y["pv"] and np.array_equal(x["hits"], y["hits"])
    for s, c in zip(slots, c0):
        assert np.array_equal(pool.counters(s), c)
    pool.close()


def test_pool_muca_refusals(gpu):
    specs = specs_of("fund", 32)
    inputs = [hot_fields(abi.make_params("fund", L=tuple(p.L[:3])), seed=95 + k, phi_mean=0.6)
              for k, (p, _, _) in enumerate(specs)]
    pool, slots = make_pool(gpu, specs, inputs, [None] * 3, False)
    w = weight_around(abi.PHISQ, 0.3)
    w.struct.checks_per_sweep = 3
    with pytest.raises(gpu.SU2GPUError, match="checks_per_sweep"):
        pool.muca_set(slots[0], w.struct)
    w = weight_around(abi.SIGMASQ, 0.3)
    with pytest.raises(gpu.SU2GPUError, match="order parameter"):
        pool.muca_set(slots[0], w.struct)
    pool.muca_set(slots[0], weight_around(abi.PHISQ, 0.3).struct)
    fields = [as_dict(f) for f in inputs]
    with pytest.raises(gpu.SU2GPUError, match="multicanonical weight"):
        pool.upload_many(slots, fields)
    with pytest.raises(gpu.SU2GPUError, match="multicanonical weight"):
        pool.cycle(slots, fields, 1)
    # the order parameter follows a single-chain upload
    f = inputs[0]
    pool.upload(slots[0], **as_dict(f))
    v = pool.calc_orderparam(slots[0], 0)
    assert abs(v - order_parameter(f, abi.PHISQ, specs[0][0].sites())) < 1e-6
    pool.close()
