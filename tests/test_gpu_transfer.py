"""Host <-> device field transfer: page-locked host arrays are converted by the
device in place (no staging copy), pageable ones through a staging buffer;
both give the same device fields and the same host arrays back, bit for bit,
for single lattices and for pools (one chain at a time or many per call)."""
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
    return {n: getattr(f, n) for n in ("link", "u1", "d0", "d1", "trip", "sing") if getattr(f, n) is not None}


def pinned_copy(gpu, f):
    out = {k: np.array(v, copy=True) for k, v in f.items()}
    for a in out.values():
        gpu.host_register(a)
    return out


def unpin(gpu, f):
    for a in f.values():
        gpu.host_unregister(a)


@pytest.mark.parametrize("content,precision", [("su2u1s", 64), ("su2u1s", 32), ("fundadj", 32), ("higgs2", 64)])
def test_pinned_equals_pageable_lattice(gpu, content, precision):
    p = abi.make_params(content, L=(8, 6, 10), precision=precision)
    f = as_dict(hot_fields(p, seed=3, phi_mean=0.5))
    a = gpu.Lattice(p, seed=1)
    a.upload(**f)
    a.run_sweeps(0, 2, graph=False)
    want = a.download()
    pf = pinned_copy(gpu, f)
    try:
        b = gpu.Lattice(p, seed=1)
        b.upload(**pf)
        b.run_sweeps(0, 2, graph=False)
        got = b.download()  # pageable output
        for n in want:
            if want[n] is not None:
                assert np.array_equal(got[n], want[n]), n
        # download into page-locked arrays (converted in place by the device)
        gpu.check(gpu.lib().su2gpu_download_fields(b.handle, *[gpu._p(pf.get(n)) for n in gpu.FIELD_NAMES]))
        for n in pf:
            assert np.array_equal(pf[n], want[n]), n
        # the host-buffer drop-in call on page-locked arrays
        c = gpu.Lattice(p, seed=1)
        host = pinned_copy(gpu, f)
        try:
            c.update_lattice_host(0, host)
            c.update_lattice_host(1, host)
            for n in host:
                assert np.array_equal(host[n], want[n]), n
        finally:
            unpin(gpu, host)
    finally:
        unpin(gpu, pf)


def test_pool_many_equals_single(gpu):
    from su2higgs_gb300 import workloads
    specs = workloads.batched_ensemble(12, seed=5)
    arena = sum(gpu.Pool.chain_bytes(p) for p, _, _ in specs)
    inputs = [workloads.hot_fields(p, seed) for p, seed, _ in specs]
    a = gpu.Pool(specs[0][0], arena_bytes=arena, max_chains=12)
    sa = [a.add(p, seed=seed, chain=chain) for p, seed, chain in specs]
    for s, f in zip(sa, inputs):
        a.upload(s, **f)
    a.run(2)
    want = [a.download(s) for s in sa]
    b = gpu.Pool(specs[0][0], arena_bytes=arena, max_chains=12)
    sb = [b.add(p, seed=seed, chain=chain) for p, seed, chain in specs]
    pinned = [pinned_copy(gpu, f) for f in inputs]
    try:
        b.upload_many(sb, pinned[:6] + inputs[6:])  # page-locked and pageable mixed
        b.run(2)
        b.download_many(sb, pinned)                 # in place
        for w, g in zip(want, pinned):
            for n in g:
                assert np.array_equal(g[n], w[n]), n
        outs = [{n: np.zeros_like(v) for n, v in f.items()} for f in inputs]
        b.download_many(sb, outs)                   # pageable
        for w, g in zip(want, outs):
            for n in g:
                assert np.array_equal(g[n], w[n]), n
    finally:
        for f in pinned:
            unpin(gpu, f)


@pytest.mark.parametrize("ring", ["1", "40000000"])
def test_pool_many_through_a_small_ring(gpu, ring, monkeypatch):
    """upload_many / download_many with a staging ring smaller than the batch
    (SU2GPU_RING_BYTES): every chain waits on the device for the chains that
    used its ring region before; the fields arrive intact both ways."""
    from su2higgs_gb300 import workloads
    monkeypatch.setenv("SU2GPU_RING_BYTES", ring)
    specs = workloads.batched_ensemble(24, seed=9)
    arena = sum(gpu.Pool.chain_bytes(p) for p, _, _ in specs)
    inputs = [workloads.hot_fields(p, seed) for p, seed, _ in specs]
    pool = gpu.Pool(specs[0][0], arena_bytes=arena, max_chains=24)
    slots = [pool.add(p, seed=seed, chain=chain) for p, seed, chain in specs]
    pinned = [pinned_copy(gpu, f) for f in inputs]
    try:
        pool.upload_many(slots, pinned)
        for s, f in zip(slots, inputs):
            got = pool.download(s)
            for n in f:
                assert np.array_equal(got[n].astype(np.float32), f[n].astype(np.float32)), n
        pool.run(1)
        want = [pool.download(s) for s in slots]
        pool.download_many(slots, pinned)
        for w, g in zip(want, pinned):
            for n in g:
                assert np.array_equal(g[n], w[n]), n
    finally:
        for f in pinned:
            unpin(gpu, f)


@pytest.mark.parametrize("ring,graph", [("", True), ("", False), ("30000000", True)])
def test_pool_cycle_equals_separate_calls(gpu, ring, graph, monkeypatch):
    """su2gpu_pool_cycle -- uploads, sweeps, measurement and downloads of
    groups of chains pipelined on three streams -- gives the fields, sums and
    counters of upload_many + run + measure + download_many bit for bit, also
    with a staging ring smaller than the batch and without graphs; twice in a
    row (the sweep counters advance)."""
    from su2higgs_gb300 import workloads
    if ring:
        monkeypatch.setenv("SU2GPU_RING_BYTES", ring)
    specs = workloads.batched_ensemble(40, seed=13)
    arena = sum(gpu.Pool.chain_bytes(p) for p, _, _ in specs)
    inputs = [workloads.hot_fields(p, seed) for p, seed, _ in specs]

    def fresh():
        pool = gpu.Pool(specs[0][0], arena_bytes=arena, max_chains=40)
        return pool, [pool.add(p, seed=seed, chain=chain) for p, seed, chain in specs]

    a, sa = fresh()
    b, sb = fresh()
    pinned = [pinned_copy(gpu, f) for f in inputs]
    outs = [{n: np.zeros_like(v) for n, v in f.items()} for f in inputs]
    try:
        for rep in range(2):
            a.upload_many(sa, inputs if rep == 0 else want_fields)
            a.run(3, graph=graph)
            want_sums = a.measure()
            want_fields = [{n: np.zeros_like(v) for n, v in f.items()} for f in inputs]
            a.download_many(sa, want_fields)
            order = list(range(len(sb)))[::-1]  # the caller's order need not be slot order
            src = pinned if rep == 0 else [outs[j] for j in range(len(sb))]
            got_sums = b.cycle([sb[j] for j in order], [src[j] for j in order], 3,
                               [outs[j] for j in order], graph=graph)
            for k, j in enumerate(order):
                assert np.array_equal(got_sums[k], want_sums[sa[j]]), (rep, j)
                for n in inputs[j]:
                    assert np.array_equal(outs[j][n], want_fields[j][n]), (rep, j, n)
        for x, y in zip(sa, sb):
            assert np.array_equal(a.counters(x), b.counters(y))
    finally:
        for f in pinned:
            unpin(gpu, f)
