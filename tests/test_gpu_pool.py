"""Pools of independent chains (the batched form) through the C ABI.

* FP64: a chain of a pool follows the trajectory of a single-lattice context
  with the same parameters, seed and chain id: the same random numbers and
  accept/reject decisions (counters equal), fields equal to rounding -- the
  per-site arithmetic is the same source compiled into two kernels, whose
  fused multiply-adds the compiler may form differently -- 1e-9 absolute
  after three sweeps and measure() sums to 1e-9 relative, as the oracle parity
  tests.  In FP32 such a rounding difference can flip an accept/reject
  decision and the two trajectories part; FP32 pool chains are checked
  statistically instead (observables of pool chains against FP64
  single-lattice chains within 3 sigma).
* Membership does not change a chain's trajectory: a chain alone and the
  same chain among others, admitted and retired around it, agree bit for bit
  (one kernel, random numbers keyed by chain and site).
* FP64 pool chains against the oracle (1e-9 after two sweeps, as the
  single-lattice parity tests).
* Admission by arena footprint; autotuning does not advance the chains;
  gradient flow of a pool chain equals the single-lattice flow.
"""
import numpy as np
import pytest

from golden_io import measure_close
from native import Oracle, hot_fields
from su2higgs_gb300 import abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from su2higgs_gb300 import gpu as g
    g.lib()
    return g


def fields_equal(a, b):
    for n in a:
        if a[n] is not None:
            d = np.abs(a[n] - b[n])
            assert np.array_equal(a[n], b[n]), (n, float(d.max()), int(np.count_nonzero(d)), d.size)


def fields_close(a, b, atol):
    for n in a:
        if a[n] is not None:
            d = np.abs(a[n] - b[n])
            assert d.max() < atol, (n, float(d.max()), int(np.count_nonzero(d)), d.size)


def chain_specs(content, precision):
    """Chains with different sizes and couplings of one recipe."""
    base = dict(precision=precision)
    return [
        (abi.make_params(content, L=(8, 8, 8), betasu2=6.0, **base), 11, 0),
        (abi.make_params(content, L=(12, 6, 10), betasu2=9.5, msq_triplet=-0.2, msq_phi=-0.05, **base), 12, 1),
        (abi.make_params(content, L=(4, 4, 4), betasu2=12.0, **base), 11, 2),
        (abi.make_params(content, L=(16, 16, 16), **base), 13, 3),
    ]


def single_run(gpu, p, f, seed, chain, nsweeps):
    lat = gpu.Lattice(p, seed=seed, chain=chain)
    lat.upload(**{k: v for k, v in f.items() if v is not None})
    lat.run_sweeps(0, nsweeps, graph=False)
    return lat.download(), lat.counters(), lat.measure()


def as_dict(f):
    return {n: getattr(f, n) for n in ("link", "u1", "d0", "d1", "trip", "sing")}


@pytest.mark.parametrize("content,precision", [("fund", 64), ("su2u1s", 64), ("higgs2", 64), ("fundadj", 64),
                                               ("adj", 64)])
@pytest.mark.parametrize("graph", [True, False])
def test_pool_chains_equal_single_lattices(gpu, content, precision, graph):
    specs = chain_specs(content, precision)
    pool = gpu.Pool(specs[0][0], arena_bytes=64 << 20, max_chains=8)
    slots, inputs = [], []
    for k, (p, seed, chain) in enumerate(specs):
        f = as_dict(hot_fields(p, seed=100 + k, phi_mean=0.5))
        s = pool.add(p, seed=seed, chain=chain)
        pool.upload(s, **f)
        slots.append(s)
        inputs.append(f)
    pool.run(2, graph=graph)
    pool.run(1, graph=graph)
    sums = pool.measure()
    atol, rtol = 1e-9, 1e-9
    for s, (p, seed, chain), f in zip(slots, specs, inputs):
        want_f, want_c, want_m = single_run(gpu, p, f, seed, chain, 3)
        fields_close(pool.download(s), want_f, atol)
        assert np.array_equal(pool.counters(s), want_c)
        ok, k, a, b = measure_close(sums[s], want_m, rtol)
        assert ok, (s, k, a, b)


def test_pool_chain_alone_equals_in_mix(gpu):
    specs = chain_specs("su2u1s", 32)
    p0, seed0, chain0 = specs[1]
    f0 = as_dict(hot_fields(p0, seed=7, phi_mean=0.5))
    alone = gpu.Pool(p0, arena_bytes=16 << 20, max_chains=4)
    s = alone.add(p0, seed=seed0, chain=chain0)
    alone.upload(s, **f0)
    alone.run(6, graph=True)
    want = alone.download(s)

    mix = gpu.Pool(p0, arena_bytes=64 << 20, max_chains=8)
    a = mix.add(specs[0][0], seed=1, chain=9)
    mix.run(1)
    t = mix.add(p0, seed=seed0, chain=chain0)
    mix.upload(t, **f0)
    mix.run(2, graph=True)
    b = mix.add(specs[3][0], seed=2, chain=8)  # membership change mid-chain
    mix.run(1, graph=True)
    mix.remove(a)
    mix.run(2, graph=False)
    mix.remove(b)
    mix.run(1, graph=True)
    fields_equal(mix.download(t), want)
    assert np.array_equal(mix.counters(t), alone.counters(s))


def test_pool_fp64_chains_match_oracle(gpu):
    specs = chain_specs("fund", 64)[:3]
    pool = gpu.Pool(specs[0][0], arena_bytes=32 << 20, max_chains=4)
    ref = []
    for k, (p, seed, chain) in enumerate(specs):
        f = hot_fields(p, seed=200 + k, phi_mean=0.5)
        s = pool.add(p, seed=seed, chain=chain)
        pool.upload(s, **as_dict(f))
        o = Oracle(p)
        o.put(f)
        for sw in range(2):
            o.set_rng(seed, sw, chain)
            o.update()
        ref.append((s, o))
    pool.run(2)
    sums = pool.measure()
    for s, o in ref:
        got, want = pool.download(s), o.get()
        for n in ("link", "d0"):
            assert np.max(np.abs(got[n] - getattr(want, n))) < 1e-9, (s, n)
        assert np.array_equal(pool.counters(s)[:22], o.counters()[:22])
        ok, k, a, b = measure_close(sums[s], o.measure(), 1e-10)
        assert ok, (s, k, a, b)


def test_pool_admission_by_footprint(gpu):
    p = abi.make_params("adj", L=(16, 16, 16), precision=32)
    per = gpu.Pool.chain_bytes(p)
    assert per == 3 * 16 * 4096 + 3 * 4 * 4096
    pool = gpu.Pool(p, arena_bytes=3 * per + per // 2, max_chains=16)
    s = [pool.add(p, seed=k) for k in range(3)]
    with pytest.raises(gpu.CapacityError):
        pool.add(p, seed=9)
    small = abi.make_params("adj", L=(8, 8, 8), precision=32)
    extra = pool.add(small, seed=10)  # the remaining half fits a smaller chain
    info = pool.info()
    assert info["chains"] == 4 and info["used_bytes"] == 3 * per + gpu.Pool.chain_bytes(small)
    pool.remove(s[1])
    s.append(pool.add(p, seed=11))  # the hole is reused
    assert pool.info()["chains"] == 4
    other = abi.make_params("fund", L=(8, 8, 8), precision=32)
    with pytest.raises(gpu.SU2GPUError):
        pool.add(other)  # a different recipe
    pool.run(2)
    assert sorted(pool.active().tolist()) == sorted([s[0], s[2], s[3], extra])
    tight = gpu.Pool(p, arena_bytes=per, max_chains=1)
    tight.add(p)
    with pytest.raises(gpu.CapacityError):
        tight.add(small)  # no free slot


def test_pool_autotune_does_not_advance(gpu):
    specs = chain_specs("su2u1s", 64)
    pool = gpu.Pool(specs[0][0], arena_bytes=64 << 20, max_chains=8)
    slots = [pool.add(p, seed=seed, chain=chain) for p, seed, chain in specs]
    pool.run(1)
    before = {s: pool.download(s) for s in slots}
    ctr = {s: pool.counters(s) for s in slots}
    choices, ms = pool.autotune()
    assert all(0 <= c < 4 for c in choices)
    for s in slots:
        fields_equal(pool.download(s), before[s])
        assert np.array_equal(pool.counters(s), ctr[s])
    pool.run(2)
    for s, (p, seed, chain) in zip(slots, specs):
        lat = gpu.Lattice(p, seed=seed, chain=chain)
        lat.run_sweeps(0, 3, graph=False)
        fields_close(pool.download(s), lat.download(), 1e-9)
        assert np.array_equal(pool.counters(s), lat.counters())


def test_pool_grad_flow_equals_lattice(gpu):
    p = abi.make_params("adj", L=(8, 8, 8), betasu2=8.0)
    f = as_dict(hot_fields(p, seed=31, phi_mean=0.3))
    pool = gpu.Pool(p, arena_bytes=8 << 20, max_chains=2)
    s = pool.add(p, seed=4)
    pool.upload(s, **f)
    lat = gpu.Lattice(p, seed=4)
    lat.upload(**{k: v for k, v in f.items() if v is not None})
    rp = pool.grad_flow(s, 0.5, 0.05, 2)
    rl = lat.grad_flow(0.5, 0.05, 2)
    assert rp.shape == rl.shape
    assert np.array_equal(rp, rl)
    fields_equal(pool.download(s), f)


def test_pool_ensemble_async_api(gpu):
    """A 64-chain slice of the batched ensemble (sides 8..48) through the
    asynchronous entry points: enqueue on a caller stream, measurement into a
    device buffer, profiled sweeps; chains still equal single lattices."""
    import torch
    from su2higgs_gb300 import workloads
    specs = workloads.batched_ensemble(64, seed=77, precision=64)
    arena = sum(gpu.Pool.chain_bytes(p) for p, _, _ in specs)
    pool = gpu.Pool(specs[0][0], arena_bytes=arena, max_chains=64)
    slots = []
    for p, seed, chain in specs:
        s = pool.add(p, seed=seed, chain=chain)
        pool.upload(s, **workloads.hot_fields(p, seed))
        slots.append(s)
    assert pool.info()["free_bytes"] == 0
    # persistent mode: the work-list kernel + the sweep-counter increment per
    # call; one launch per pass otherwise (what the automatic mode picks for
    # these 64 chains, 8k tiles per pass)
    pool.persistent = True
    assert pool.launches_per_sweep() == 2
    pool.persistent = False
    assert pool.launches_per_sweep() == 6 + 10 + 1
    pool.persistent = None
    assert pool.launches_per_sweep() == 6 + 10 + 1
    stream = torch.cuda.Stream()
    sums = torch.zeros((64, abi.NMEAS), dtype=torch.float64, device="cuda")
    pool.set_stream(stream.cuda_stream)
    with torch.cuda.stream(stream):
        pool.enqueue(2, graph=True)
        assert pool.enqueue_measure(sums.data_ptr(), 64) == 64
    stream.synchronize()
    pool.set_stream(None)
    pool.run(0)
    kinds, ms = pool.profile_sweep()
    assert sorted(set(kinds.tolist())) == [0, 3] and len(kinds) == 16 and np.all(ms > 0)
    host_sums = pool.measure()
    dev = sums.cpu().numpy()
    for k in range(0, 64, 8):
        p, seed, chain = specs[k]
        lat = gpu.Lattice(p, seed=seed, chain=chain)
        lat.upload(**workloads.hot_fields(p, seed))
        lat.run_sweeps(0, 2, graph=True)
        ok, i, a, b = measure_close(dev[k], lat.measure(), 1e-9)
        assert ok, (k, i, a, b)
        lat.run_sweeps(2, 1, graph=False)
        fields_close(pool.download(slots[k]), lat.download(), 1e-9)
        assert np.array_equal(pool.counters(slots[k]), lat.counters())
        ok, i, a, b = measure_close(host_sums[slots[k]], lat.measure(), 1e-9)
        assert ok, (k, i, a, b)


def test_pool_fp32_samples_the_fp64_distribution(gpu):
    """FP32 pool chains (fundamental Higgs, 8^3, beta 8, m^2 -0.1, lambda 0.002)
    against FP64 single-lattice chains: plaquette, phi^2 and the hopping term
    agree within 3 sigma of binned jackknife errors."""
    from stats import compare_means
    p32 = abi.make_params("fund", L=(8, 8, 8), precision=32)
    p64 = abi.make_params("fund", L=(8, 8, 8), precision=64)
    nchains, ntherm, nmeas = 4, 200, 3000
    pool = gpu.Pool(p32, arena_bytes=8 << 20, max_chains=nchains)
    slots = []
    for k in range(nchains):
        s = pool.add(p32, seed=500 + k, chain=k)
        f = as_dict(hot_fields(p32, seed=600 + k, phi_mean=1.0))
        pool.upload(s, **{n: v for n, v in f.items() if v is not None})
        slots.append(s)
    pool.run(ntherm)
    V = p32.sites()
    obs32 = {s: [] for s in slots}
    for _ in range(nmeas):
        pool.run(1)
        for s, m in pool.measure().items():
            obs32[s].append((m[abi.M_WILSON] / (V * p32.betasu2), m[abi.M_PHI2] / V, m[abi.M_COV_PHI] / (3 * V)))
    obs64 = []
    for k in range(nchains):
        lat = gpu.Lattice(p64, seed=700 + k, chain=k)
        f = as_dict(hot_fields(p64, seed=600 + k, phi_mean=1.0))
        lat.upload(**{n: v for n, v in f.items() if v is not None})
        lat.run_sweeps(0, ntherm, graph=True)
        rows = []
        for sw in range(nmeas):
            lat.update_lattice(ntherm + sw)
            m = lat.measure()
            rows.append((m[abi.M_WILSON] / (V * p64.betasu2), m[abi.M_PHI2] / V, m[abi.M_COV_PHI] / (3 * V)))
        obs64.append(np.array(rows))
    a = np.concatenate([np.array(obs32[s]) for s in slots])
    b = np.concatenate(obs64)
    for k, name in enumerate(("plaquette", "phi2", "hopping")):
        z, ma, mb = compare_means(a[:, k], b[:, k])
        assert z < 3.0, (name, z, ma, mb)
