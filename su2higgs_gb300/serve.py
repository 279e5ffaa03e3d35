"""Served stream of Monte Carlo chains with continuous batching.

A request is one independent chain of the su2higgs update sweep: lattice side,
field content, couplings, a number of sweeps and, optionally, a gradient-flow
measurement at the end.  The reference runs one chain per process
(su2higgs main loop, main.c:302-379); here chains of many requests share the GPU:

* one pool (su2gpu_pool_*) per field content keeps the admitted chains
  resident in a device arena; a chain is admitted when its fields fit in the
  arena (HBM footprint) and a slot is free, in arrival order, with smaller
  requests allowed past one that does not fit (backfill);
* the server works in rounds: every pool runs a quantum of sweeps -- the
  smaller of `quantum` and the fewest sweeps any of its chains still owes,
  so no chain runs past its request -- as CUDA-graph replays on its own
  stream, the pools' quanta overlapping on the device; requests that arrived
  meanwhile are admitted at the next round as slots and memory free up;
* a chain that is done is measured (measure() sums), and when it asked for a
  gradient flow, copied out of its pool into a context of its own whose flow
  (gradflow.c:46-173) runs on a worker thread while the pools go on.

A chain's results do not depend on the other chains or on the quanta: its
random numbers are keyed by its seed, chain id, sweep and site.

A chain starts cold -- unit links, zero U(1) angles and scalars (setfields,
init.c:92-110, with the initial scalar values phi0 = sigma0 = singlet0 = 0),
so no host field traffic is needed to admit it -- unless its request carries
a starting configuration (`start`: FP64 host fields in the reference's
lattice-file layout, as a loaded checkpoint, load_lattice checkpoint.c:133-214),
which is uploaded into the chain's slot when it is admitted.
"""
import collections
import concurrent.futures
import dataclasses
import time

import numpy as np

from . import abi

CONTENTS = ("fund", "adj", "su2u1s")
SIDES = (16, 32, 64, 96, 128)
SWEEPS = (500, 5000)
FLOW_FRACTION = 0.3
# gradient flow of a request that carries one: flow time 0..4, step 0.01
FLOW = dict(t_max=4.0, dt=0.01, meas_interval=10)
# coupling ranges of the workloads (beta_G, the scalar mass term)
BETA = (6.0, 12.0)
MSQ = (-0.3, 0.1)


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float  # seconds after the start of the stream
    content: str
    L: int
    sweeps: int
    flow: bool
    betasu2: float
    msq: float
    seed: int
    # optional starting configuration: {field name: FP64 host array} (names
    # link, u1, d0, d1, trip, sing; absent fields start cold)
    start: dict = None

    def params(self, precision=32):
        kw = dict(precision=precision, betasu2=self.betasu2)
        if self.content == "adj":
            kw.update(msq_triplet=self.msq, b4=0.005)
        else:
            kw.update(msq_phi=self.msq)
        return abi.make_params(self.content, L=(self.L,) * 3, **kw)


@dataclasses.dataclass
class Result:
    rid: int
    arrival: float
    admitted: float
    finished: float
    sites: int
    sweeps: int
    sums: np.ndarray
    counters: np.ndarray
    flow_rows: np.ndarray = None

    @property
    def latency(self):
        return self.finished - self.arrival


def make_stream(rate, duration, seed=1, sides=SIDES, sweeps=SWEEPS, flow_fraction=FLOW_FRACTION,
                contents=CONTENTS):
    """Poisson arrivals at `rate` per second over `duration` seconds; each
    request draws its side, content, couplings, sweep count and flow flag."""
    rng = np.random.default_rng(seed)
    out, t, rid = [], 0.0, 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        out.append(Request(rid=rid, arrival=t, content=str(rng.choice(contents)), L=int(rng.choice(sides)),
                           sweeps=int(rng.integers(sweeps[0], sweeps[1] + 1)),
                           flow=bool(rng.random() < flow_fraction), betasu2=float(rng.uniform(*BETA)),
                           msq=float(rng.uniform(*MSQ)), seed=int(rng.integers(1, 2 ** 62))))
        rid += 1
    return out


class _Live:
    __slots__ = ("req", "slot", "remaining", "admitted", "params")

    def __init__(self, req, slot, admitted, params):
        self.req, self.slot, self.remaining, self.admitted, self.params = req, slot, req.sweeps, admitted, params


class Server:
    """Continuous batching over one pool per field content.

    `pool_factory(recipe, arena_bytes, max_chains)` makes a pool (gpu.Pool or
    a stand-in with the same methods); `chain_bytes(params)` gives a chain's
    arena footprint.  `arena_bytes` is the device budget of each content's
    pool."""

    def __init__(self, pool_factory, chain_bytes, arena_bytes, max_chains=512, precision=32, quantum=100,
                 flow=FLOW, clock=time.perf_counter, sleep=time.sleep, graph=True, flow_workers=1):
        self.precision = precision
        self.quantum = quantum
        self.flow = flow
        self.clock = clock
        self.sleep = sleep
        self.graph = graph
        self.chain_bytes = chain_bytes
        self.arena_bytes = arena_bytes
        self.pools = {}
        self._factory = pool_factory
        self.max_chains = max_chains
        self.waiting = collections.deque()
        self.live = {c: {} for c in CONTENTS}  # content -> slot -> _Live
        self.results = {}
        self.site_updates = 0
        self._flows = concurrent.futures.ThreadPoolExecutor(max_workers=flow_workers)
        self._pending_flows = []
        self.t0 = None

    def now(self):
        return self.clock() - self.t0

    def pool(self, content):
        if content not in self.pools:
            recipe = abi.make_params(content, L=(8, 8, 8), precision=self.precision)
            self.pools[content] = self._factory(recipe, self.arena_bytes, self.max_chains)
        return self.pools[content]

    def submit(self, req):
        if self.chain_bytes(req.params(self.precision)) > self.arena_bytes:
            raise ValueError(f"request {req.rid} needs more than the whole arena")
        self.waiting.append(req)

    def admit(self):
        """Admit waiting requests in arrival order while they fit; a request
        that does not fit stays at its place and later ones may pass it."""
        from .gpu import CapacityError
        still = collections.deque()
        t = self.now()
        while self.waiting:
            req = self.waiting.popleft()
            p = req.params(self.precision)
            pool = self.pool(req.content)
            try:
                slot = pool.add(p, seed=req.seed, chain=req.rid)
            except CapacityError:
                still.append(req)
                continue
            if req.start:
                pool.upload(slot, **req.start)
            self.live[req.content][slot] = _Live(req, slot, t, p)
        self.waiting = still

    def round(self):
        """Admit, run one quantum of every pool, retire finished chains.
        Returns the number of sweeps run by the largest quantum."""
        self.admit()
        quanta = {}
        for content, chains in self.live.items():
            if not chains:
                continue
            q = min(self.quantum, min(c.remaining for c in chains.values()))
            self.pools[content].enqueue(q, self.graph)
            quanta[content] = q
        for content, q in quanta.items():
            self.pools[content].run(0)  # waits for the quantum, surfaces kernel errors
            for c in self.live[content].values():
                c.remaining -= q
                self.site_updates += q * c.params.sites()
        for content in quanta:
            self._retire(content)
        self._collect_flows(block=False)
        return max(quanta.values(), default=0)

    def _retire(self, content):
        chains = self.live[content]
        done = [c for c in chains.values() if c.remaining == 0]
        if not done:
            return
        pool = self.pools[content]
        sums = pool.measure()
        t = self.now()
        for c in done:
            r = Result(rid=c.req.rid, arrival=c.req.arrival, admitted=c.admitted, finished=t,
                       sites=c.params.sites(), sweeps=c.req.sweeps, sums=sums[c.slot],
                       counters=pool.counters(c.slot))
            if c.req.flow:
                lat = pool.extract(c.slot)
                fut = self._flows.submit(self._run_flow, lat)
                self._pending_flows.append((r, fut))
            else:
                self.results[r.rid] = r
            pool.remove(c.slot)
            del chains[c.slot]

    def _run_flow(self, lat):
        try:
            return lat.grad_flow(self.flow["t_max"], self.flow["dt"], self.flow["meas_interval"])
        finally:
            lat.close()

    def _collect_flows(self, block):
        keep = []
        for r, fut in self._pending_flows:
            if block or fut.done():
                r.flow_rows = fut.result()
                r.finished = self.now()
                self.results[r.rid] = r
            else:
                keep.append((r, fut))
        self._pending_flows = keep

    def busy(self):
        return bool(self.waiting) or any(self.live.values()) or bool(self._pending_flows)

    def serve(self, stream, deadline=None, idle_sleep=0.001):
        """Play `stream` in real time (by `clock`): a request joins the queue
        once the clock passes its arrival time.  Stops when every request is
        done or at `deadline` seconds; returns the results by request id."""
        self.t0 = self.clock()
        pending = collections.deque(sorted(stream, key=lambda r: r.arrival))
        while pending or self.busy():
            t = self.now()
            if deadline is not None and t >= deadline:
                break
            while pending and pending[0].arrival <= t:
                self.submit(pending.popleft())
            if any(self.live.values()) or self.waiting:
                self.round()
                continue
            # nothing on the GPU: wait for the next arrival or a running flow
            self._collect_flows(block=False)
            if pending:
                self.sleep(max(0.0, min(pending[0].arrival - self.now(), 0.05)))
            elif self._pending_flows:
                self.sleep(idle_sleep)
        if deadline is None:
            self._collect_flows(block=True)
        self.unfinished = (len(pending) + len(self.waiting) + sum(len(v) for v in self.live.values())
                           + len(self._pending_flows))
        return self.results

    def close(self):
        self._flows.shutdown(wait=True)
        for p in self.pools.values():
            p.close()
        self.pools = {}


def summarize(results, wall, site_updates):
    lat = np.array([r.latency for r in results.values()]) if results else np.zeros(1)
    return {"completed": len(results), "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)), "mean_latency_s": float(lat.mean()),
            "site_updates_per_s": site_updates / wall if wall > 0 else 0.0, "wall_s": wall}
