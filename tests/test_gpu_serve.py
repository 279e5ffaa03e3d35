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
