"""Host logic of the served stream (su2higgs_gb300/serve.py) on the CPU: a
stand-in pool with the gpu.Pool interface counts sweeps and arena bytes, and a
simulated clock advances with the work, so admission, backfill, quanta,
retirement and the flow hand-off are checked without a GPU."""
import numpy as np
import pytest

from su2higgs_gb300 import abi, serve
from su2higgs_gb300.gpu import CapacityError


class Clock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def advance(self, dt):
        self.t += dt


def footprint(p):
    return p.sites() * 4 * (12 + 4)  # any monotone footprint will do


class FakeLattice:
    def __init__(self, sweeps):
        self.sweeps = sweeps
        self.closed = False

    def grad_flow(self, t_max, dt, meas_interval):
        n = int(round(t_max / dt)) // meas_interval + 1
        rows = np.zeros((n, 1 + abi.NMEAS))
        rows[:, 0] = np.arange(n) * dt * meas_interval
        rows[:, 1] = self.sweeps
        return rows

    def close(self):
        self.closed = True


class FakePool:
    cost_per_site_sweep = 1e-9  # simulated seconds

    def __init__(self, recipe, arena_bytes, max_chains, clock, log):
        self.recipe, self.arena, self.max_chains, self.clock, self.log = recipe, arena_bytes, max_chains, clock, log
        self.chains = {}  # slot -> [params, sweeps done, seed, chain]
        self.pending = 0

    def used(self):
        return sum(footprint(c[0]) for c in self.chains.values())

    def add(self, p, seed=0, chain=0):
        assert p.content == self.recipe.content and p.precision == self.recipe.precision
        if len(self.chains) >= self.max_chains or self.used() + footprint(p) > self.arena:
            raise CapacityError("full")
        slot = min(set(range(self.max_chains)) - set(self.chains))
        self.chains[slot] = [p, 0, seed, chain]
        self.log.append(("add", chain, self.clock()))
        return slot

    def upload(self, slot, **fields):
        self.log.append(("upload", self.chains[slot][3], tuple(sorted(fields))))

    def remove(self, slot):
        self.log.append(("remove", self.chains[slot][3], self.clock()))
        del self.chains[slot]

    def enqueue(self, q, graph=True):
        for c in self.chains.values():
            c[1] += q
        self.pending += q * sum(c[0].sites() for c in self.chains.values()) * self.cost_per_site_sweep
        self.log.append(("quantum", q, len(self.chains)))

    def run(self, n, graph=True):
        assert n == 0
        self.clock.advance(self.pending)
        self.pending = 0

    def measure(self):
        return {s: np.full(abi.NMEAS, float(c[1])) for s, c in self.chains.items()}

    def counters(self, slot):
        return np.full(abi.NCOUNTERS, self.chains[slot][1], dtype=np.int64)

    def extract(self, slot):
        return FakeLattice(self.chains[slot][1])

    def close(self):
        pass


def make_server(arena, quantum=100, max_chains=64):
    clock = Clock()
    log = []
    srv = serve.Server(lambda r, a, m: FakePool(r, a, m, clock, log), footprint, arena, max_chains=max_chains,
                       quantum=quantum, clock=clock, sleep=clock.advance)
    return srv, clock, log


def test_every_request_completes_with_its_sweeps():
    stream = serve.make_stream(rate=20, duration=3.0, seed=5, sides=(8, 12, 16), sweeps=(50, 400))
    srv, clock, log = make_server(arena=8 * footprint(abi.make_params("fund", L=(16, 16, 16))), quantum=64)
    res = srv.serve(stream)
    srv.close()
    assert srv.unfinished == 0
    assert sorted(res) == [r.rid for r in stream]
    for r in stream:
        out = res[r.rid]
        assert out.sums[0] == r.sweeps  # the chain ran exactly its sweeps
        assert out.counters[0] == r.sweeps
        assert (out.flow_rows is not None) == r.flow
        if r.flow:
            assert out.flow_rows.shape == (41, 1 + abi.NMEAS) and np.all(out.flow_rows[:, 1] == r.sweeps)
        assert out.arrival <= out.admitted <= out.finished
    # quanta never exceed the requested quantum
    assert max(q for kind, q, n in log if kind == "quantum") <= 64
    assert srv.site_updates == sum(r.sweeps * r.L ** 3 for r in stream)


def test_admission_by_footprint_and_backfill():
    big = abi.make_params("fund", L=(16, 16, 16))
    arena = 2 * footprint(big) + footprint(abi.make_params("fund", L=(8, 8, 8)))
    reqs = [serve.Request(rid=k, arrival=0.0, content="fund", L=L, sweeps=200, flow=False, betasu2=8.0,
                          msq=-0.1, seed=k + 1)
            for k, L in enumerate((16, 16, 16, 8))]
    srv, clock, log = make_server(arena, quantum=1000)
    res = srv.serve(reqs)
    srv.close()
    adds = [(c, t) for kind, c, t in log if kind == "add"]
    # the third 16^3 chain has to wait; the 8^3 chain is admitted past it
    assert [c for c, _ in adds[:3]] == [0, 1, 3]
    assert adds[3][0] == 2 and adds[3][1] > 0.0
    assert res[2].admitted > res[3].admitted
    with pytest.raises(ValueError):
        srv2, _, _ = make_server(footprint(big) - 1)
        srv2.submit(reqs[0])


def test_results_do_not_depend_on_the_mix():
    """The same request alone and inside a stream: same sweeps, same chain id
    and seed handed to the pool (the GPU test checks the fields)."""
    stream = serve.make_stream(rate=50, duration=1.0, seed=9, sides=(8, 16), sweeps=(30, 300))
    target = stream[len(stream) // 2]
    srv, _, log = make_server(arena=4 * footprint(abi.make_params("fund", L=(16, 16, 16))), quantum=50)
    mix = srv.serve(stream)
    srv.close()
    alone_srv, _, _ = make_server(arena=4 * footprint(abi.make_params("fund", L=(16, 16, 16))), quantum=50)
    alone = alone_srv.serve([target])
    alone_srv.close()
    assert np.array_equal(mix[target.rid].sums, alone[target.rid].sums)


def test_deadline_leaves_work_unfinished():
    stream = serve.make_stream(rate=100, duration=2.0, seed=3, sides=(32,), sweeps=(4000, 5000))
    srv, clock, log = make_server(arena=2 * footprint(abi.make_params("fund", L=(32, 32, 32))), quantum=100)
    res = srv.serve(stream, deadline=1.0)
    srv.close()
    assert srv.unfinished > 0 and len(res) + srv.unfinished == len(stream)


def test_stream_statistics():
    s = serve.make_stream(rate=20, duration=600, seed=1)
    assert abs(len(s) / 600 - 20) < 0.5
    gaps = np.diff([r.arrival for r in s])
    assert abs(gaps.mean() - 0.05) < 0.003 and abs(gaps.std() / gaps.mean() - 1) < 0.05  # exponential
    assert set(r.content for r in s) == set(serve.CONTENTS)
    assert set(r.L for r in s) == set(serve.SIDES)
    assert 0.27 < np.mean([r.flow for r in s]) < 0.33
    assert min(r.sweeps for r in s) >= 500 and max(r.sweeps for r in s) <= 5000


def test_requests_with_a_starting_configuration_are_uploaded_at_admission():
    stream = serve.make_stream(rate=20, duration=1.0, seed=9, sides=(8,), sweeps=(50, 60), flow_fraction=0.0)
    start = {"link": np.zeros((512, 3, 4))}
    stream = [serve.Request(**{**r.__dict__, "start": start if r.rid % 2 == 0 else None}) for r in stream]
    srv, clock, log = make_server(arena=1 << 30)
    res = srv.serve(stream)
    srv.close()
    assert sorted(res) == [r.rid for r in stream]
    uploads = [e for e in log if e[0] == "upload"]
    assert sorted(e[1] for e in uploads) == [r.rid for r in stream if r.rid % 2 == 0]
    assert all(e[2] == ("link",) for e in uploads)
    # each upload comes right after its chain's admission
    for k, e in enumerate(log):
        if e[0] == "upload":
            assert log[k - 1][0] == "add" and log[k - 1][1] == e[1]
