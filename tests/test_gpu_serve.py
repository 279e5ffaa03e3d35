"""The served stream on the GPU: each request's results (measure() sums,
counters, gradient-flow rows) are the same when it runs alone and when it runs
in a mix of requests that arrive while others are on the device (bit for bit:
one kernel per content, random numbers keyed by the request's seed and chain
id, not by its slot or its neighbours)."""
import numpy as np
import pytest

from su2higgs_gb300 import serve

pytestmark = pytest.mark.gpu

FLOW = dict(t_max=0.2, dt=0.02, meas_interval=2)


def make(gpu, quantum):
    return serve.Server(gpu.Pool, gpu.Pool.chain_bytes, arena_bytes=32 << 20, max_chains=32, quantum=quantum,
                        flow=FLOW)


def test_served_results_alone_equal_in_mix():
    from su2higgs_gb300 import gpu
    gpu.lib()
    stream = serve.make_stream(rate=400, duration=0.1, seed=21, sides=(8, 12, 16), sweeps=(20, 90),
                               flow_fraction=0.4)
    assert len(stream) >= 20 and {r.content for r in stream} == set(serve.CONTENTS)
    srv = make(gpu, quantum=16)
    mix = srv.serve(stream)
    srv.close()
    assert srv.unfinished == 0 and sorted(mix) == [r.rid for r in stream]
    # requests overlapped on the device: some were admitted before others finished
    assert any(a.admitted < b.finished and b.admitted < a.finished
               for a in mix.values() for b in mix.values() if a.rid != b.rid)
    picks = [r for r in stream if r.flow][:2] + [r for r in stream if not r.flow][:3]
    for r in picks:
        alone_srv = make(gpu, quantum=7)  # other quanta too
        alone = alone_srv.serve([serve.Request(**{**r.__dict__, "arrival": 0.0})])[r.rid]
        alone_srv.close()
        m = mix[r.rid]
        assert np.array_equal(alone.sums, m.sums), r
        assert np.array_equal(alone.counters, m.counters), r
        if r.flow:
            assert alone.flow_rows.shape[0] >= 6
            assert np.array_equal(alone.flow_rows, m.flow_rows), r
        else:
            assert alone.flow_rows is None and m.flow_rows is None
        assert np.all(np.isfinite(m.sums)) and m.counters[0] == r.sweeps * 3 * r.L ** 3


def test_served_request_with_a_starting_configuration():
    """A request that carries its starting fields gives the same results as
    a pool chain uploaded with them and run alone (and different results from
    the cold start)."""
    from native import hot_fields
    from su2higgs_gb300 import gpu
    gpu.lib()
    r0 = serve.make_stream(rate=100, duration=0.2, seed=33, sides=(8,), sweeps=(30, 30), flow_fraction=0.0)[0]
    p = r0.params(32)
    f = hot_fields(p, seed=77, phi_mean=0.5)
    start = {n: getattr(f, n) for n in ("link", "u1", "d0", "d1", "trip", "sing") if getattr(f, n) is not None}
    req = serve.Request(**{**r0.__dict__, "arrival": 0.0, "start": start})
    srv = make(gpu, quantum=8)
    got = srv.serve([req])[req.rid]
    srv.close()
    pool = gpu.Pool(p, arena_bytes=16 << 20, max_chains=2)
    slot = pool.add(p, seed=req.seed, chain=req.rid)
    pool.upload(slot, **start)
    pool.run(req.sweeps)
    want = pool.measure()[slot]
    pool.close()
    assert np.array_equal(got.sums, want)
    cold_srv = make(gpu, quantum=8)
    cold = cold_srv.serve([serve.Request(**{**r0.__dict__, "arrival": 0.0})])[req.rid]
    cold_srv.close()
    assert not np.array_equal(cold.sums, got.sums)
