"""Parity of the CUDA path (through the C ABI) with the reference's own outputs
(golden fixtures) and with the oracle, for the plain FP64 path.

Tolerances (the reference computes in FP64, with long double in polysolve3 and
local_su2wilson; the GPU in FP64 with fused multiply-adds):
  * layout tables: bit-exact
  * deterministic sums / per-site quantities: 1e-12 relative
  * fields after one stochastic sweep: 1e-11 absolute (same uniforms, same
    accept/reject decisions; rounding differences only), 1e-9 after three
  * accept/reject counters: exact
"""
import numpy as np
import pytest

from golden_io import fields_of, load, measure_close, names, params_of, weight_of
from native import Oracle, hot_fields, ref_sums_to_layout
from su2higgs_gb300 import abi

pytestmark = pytest.mark.gpu

RTOL = 1e-12
ATOL1 = 1e-11
ATOL3 = 1e-9


@pytest.fixture(scope="module")
def gpu():
    from su2higgs_gb300 import gpu as g
    g.lib()
    return g


def upload(lat, f):
    lat.upload(link=f.link, u1=f.u1, d0=f.d0, d1=f.d1, trip=f.trip, sing=f.sing)


def max_diff(got, want):
    out = {}
    for n in ("link", "u1", "d0", "d1", "trip", "sing"):
        w = getattr(want, n)
        if w is not None:
            out[n] = float(np.max(np.abs(got[n] - w)))
    return out


@pytest.mark.parametrize("name", names("layout_"))
def test_layout_tables(gpu, name):
    d = load(name)
    L = tuple(int(x) for x in d["L"])
    lat = gpu.Lattice(abi.make_params("pure", L=L))
    nx, pv, co, par = lat.layout_tables()
    assert np.array_equal(nx, d["next"])
    assert np.array_equal(pv, d["prev"])
    assert np.array_equal(co, d["coords"])
    assert np.array_equal(par, d["parity"])


def test_layout_table_digests(gpu):
    """The device's closed-form layout of the larger sides (24^3 ... 128^3)
    against the SHA-256 of the reference's own layout() tables."""
    from native import layout_digest
    d = load("tables_sha256.npz")
    for L, digest in zip(d["L"], d["sha256"]):
        lat = gpu.Lattice(abi.make_params("pure", L=tuple(int(x) for x in L)))
        assert layout_digest(*lat.layout_tables()) == str(digest), tuple(L)
        lat.close()


# per-site values: (fixture key, vector width or 0 for a scalar).  A
# vector value (a staple of one direction, a proposed doublet or triplet) is
# compared relative to its own length at that site, a scalar relative to
# itself.
SITE_KEYS = [("link_staple", 4), ("wilson_staple", 4), ("localact_su2link", 0), ("localact_u1link", 0),
             ("staple_doublet", 4), ("localact_doublet", 0), ("localact_singlet", 0), ("or_doublet", 4),
             ("or_doublet1", 4), ("or_triplet", 3), ("or_singlet", 0)]


def site_rel_err(got, want, width):
    if not width:
        from native import rel_err
        return rel_err(got, want)
    g = np.asarray(got).reshape(-1, width)
    w = np.asarray(want).reshape(-1, width)
    return float(np.max(np.max(np.abs(g - w), axis=1) / np.maximum(np.linalg.norm(w, axis=1), 1e-300)))


@pytest.mark.parametrize("name", names("sites_"))
def test_site_values_match_reference(gpu, name):
    """Staples, local actions and overrelaxation proposals of every site,
    computed on the device by the functions the update kernels call, on a
    configuration of the reference's own run: within 1e-12 relative of the
    reference's FP64 values (staples.c:84-302, su2u1.c:166-723,
    overrelax.c:54-417).  The proposals come from the cubic root of
    polysolve3, which the reference takes by Cardano's formula in long
    double and the device refines by a Newton step to the root itself: the
    reference's own root is up to ~5e-12 (relative) from the exact one where
    the formula cancels, which moves a proposed field by ~4e-13 of its length
    at most on these configurations."""
    d = load(name)
    p = params_of(d)
    lat = gpu.Lattice(p)
    upload(lat, fields_of(d, p, "in_"))
    checked = 0
    for key, width in SITE_KEYS:
        if key not in d:
            continue
        got = lat.site_values(key)
        err = site_rel_err(got, d[key], width)
        print(f"{name} {key}: max relative difference {err:.2e}")
        assert err < RTOL, (key, err)
        checked += 1
    assert checked >= 3
    # the fields are unchanged by the overrelaxation probes
    for k, v in max_diff(lat.download(), fields_of(d, p, "in_")).items():
        assert v == 0.0, k


def test_upload_download_roundtrip(gpu):
    p = abi.make_params("su2u1s", L=(6, 4, 8))
    f = hot_fields(p, seed=5)
    lat = gpu.Lattice(p)
    upload(lat, f)
    got = lat.download()
    assert all(v == 0.0 for v in max_diff(got, f).values())


@pytest.mark.parametrize("name", names("sites_"))
def test_measure_matches_reference(gpu, name):
    d = load(name)
    p = params_of(d)
    lat = gpu.Lattice(p)
    upload(lat, fields_of(d, p, "in_"))
    ok, k, a, b = measure_close(lat.measure(), d["measure"], RTOL)
    assert ok, (k, a, b)


@pytest.mark.parametrize("name", names("sweep_"))
def test_sweeps_match_reference(gpu, name):
    d = load(name)
    p = params_of(d)
    seed, s0 = int(d["seed"]), int(d["first_sweep"])
    lat = gpu.Lattice(p, seed=seed)
    upload(lat, fields_of(d, p, "in_"))
    lat.update_lattice(s0)
    for k, v in max_diff(lat.download(), fields_of(d, p, "out1_")).items():
        assert v < ATOL1, (k, v)
    assert np.array_equal(lat.counters()[:22], d["counters1"][:22])
    lat.update_lattice(s0 + 1)
    lat.update_lattice(s0 + 2)
    for k, v in max_diff(lat.download(), fields_of(d, p, "out3_")).items():
        assert v < ATOL3, (k, v)
    assert np.array_equal(lat.counters()[:22], d["counters3"][:22])
    ok, k, a, b = measure_close(lat.measure(), d["measure3"], 1e-8)
    assert ok, (k, a, b)


@pytest.mark.parametrize("name", names("muca_"))
def test_multicanonical_matches_reference(gpu, name):
    d = load(name)
    p = params_of(d)
    seed = int(d["seed"])
    lat = gpu.Lattice(p, seed=seed)
    upload(lat, fields_of(d, p, "in_"))
    w = weight_of(d, "w0_")
    lat.muca_set(w.struct)
    for s in range(int(d["nsweeps"])):
        lat.update_lattice(100 + s)
    for k, v in max_diff(lat.download(), fields_of(d, p, "out_")).items():
        assert v < ATOL3, (k, v)
    assert np.array_equal(lat.counters()[:22], d["counters"][:22])
    w1 = weight_of(d, "w1_")
    lat.muca_get(w.struct)
    assert np.array_equal(w.hits, w1.hits)
    assert np.max(np.abs(w.W - w1.W)) < 1e-9
    assert w.struct.last_max == w1.struct.last_max
    assert w.struct.muca_count == w1.struct.muca_count
    assert abs(w.struct.delta - w1.struct.delta) < 1e-15
    assert np.allclose(list(w.struct.param_value), list(w1.struct.param_value), rtol=1e-9, atol=0)
    if w.struct.mode == abi.MUCA_SLOW:  # update_weight_slow's accumulators
        assert np.array_equal(w.gsum, w1.gsum) and np.array_equal(w.nsum, w1.nsum)
        assert np.allclose(w.hgram, w1.hgram, rtol=1e-9, atol=0)


@pytest.mark.parametrize("name", names("flow_"))
def test_gradient_flow_matches_reference(gpu, name):
    d = load(name)
    p = params_of(d)
    lat = gpu.Lattice(p)
    upload(lat, fields_of(d, p, "in_"))
    rows = lat.grad_flow(float(d["t_max"]), float(d["dt"]), int(d["meas_interval"]))
    ref = d["rows_raw"]
    assert rows.shape[0] == ref.shape[0]
    for r_g, r_r in zip(rows, ref):
        ok, k, a, b = measure_close(r_g[1:], ref_sums_to_layout(p, r_r), RTOL)
        assert ok, (k, a, b)
    # the flow works on a copy: the lattice itself is unchanged
    for k, v in max_diff(lat.download(), fields_of(d, p, "in_")).items():
        assert v == 0.0, k


@pytest.mark.parametrize("content,L", [("fund", (16, 16, 16)), ("su2u1s", (12, 8, 16)), ("adj", (8, 12, 10))])
def test_larger_lattice_matches_oracle(gpu, content, L):
    p = abi.make_params(content, L=L)
    f = hot_fields(p, seed=41, phi_mean=0.5)
    lat = gpu.Lattice(p, seed=77)
    upload(lat, f)
    o = Oracle(p)
    o.put(f)
    for s in (9, 10):
        lat.update_lattice(s)
        o.set_rng(77, s)
        o.update()
    for k, v in max_diff(lat.download(), o.get()).items():
        assert v < ATOL3, (k, v)
    assert np.array_equal(lat.counters()[:22], o.counters()[:22])
    ok, k, a, b = measure_close(lat.measure(), o.measure(), 1e-10)
    assert ok, (k, a, b)


def test_graph_replay_equals_stepwise(gpu):
    p = abi.make_params("su2u1s", L=(8, 8, 8))
    f = hot_fields(p, seed=3, phi_mean=0.5)
    a = gpu.Lattice(p, seed=99)
    b = gpu.Lattice(p, seed=99)
    upload(a, f)
    upload(b, f)
    for s in range(20, 25):
        a.update_lattice(s)
    b.run_sweeps(20, 5, graph=True)
    fa, fb = a.download(), b.download()
    for n in fa:
        if fa[n] is not None:
            assert np.array_equal(fa[n], fb[n]), n
    assert np.array_equal(a.counters(), b.counters())


def test_host_buffer_dropin_equals_resident(gpu):
    p = abi.make_params("fund", L=(8, 8, 8))
    f = hot_fields(p, seed=8, phi_mean=0.5)
    a = gpu.Lattice(p, seed=5)
    upload(a, f)
    a.update_lattice(1)
    ga = a.download()
    b = gpu.Lattice(p, seed=5)
    host = {"link": f.link.copy(), "d0": f.d0.copy()}
    b.update_lattice_host(1, host)
    assert np.array_equal(ga["link"], host["link"])
    assert np.array_equal(ga["d0"], host["d0"])


def test_calc_orderparam(gpu):
    p = abi.make_params("fund", L=(8, 8, 8))
    f = hot_fields(p, seed=9, phi_mean=0.5)
    lat = gpu.Lattice(p)
    upload(lat, f)
    from native import WeightBuf
    w = WeightBuf(8)
    w.pos[:] = np.linspace(-1, 1, 10)
    w.linearize()
    s = w.struct
    s.min, s.max = -1.0, 1.0
    lat.muca_set(s)
    half = p.sites() // 2
    ev = lat.calc_orderparam(0)
    tot = lat.calc_orderparam(1)
    ph = 0.5 * np.sum(f.d0 ** 2, axis=1)
    assert abs(tot - ph.sum() / p.sites()) < 1e-13
    assert abs(ev - (ph[:half].sum() / p.sites())) < 1e-13


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("content", ["su2u1s", "adj"])
def test_launch_variants_bit_identical(gpu, content, precision):
    """The random stream is keyed by site, not by thread or block, so every
    launch shape the autotuner may pick produces the same fields bit for bit."""
    p = abi.make_params(content, L=(12, 8, 10), precision=precision)
    f = hot_fields(p, seed=21, phi_mean=0.5)
    ref = None
    for v in range(4):
        lat = gpu.Lattice(p, seed=8)
        upload(lat, f)
        lat.set_variants([v] * 5)
        lat.run_sweeps(0, 3, graph=False)
        got = lat.download()
        if ref is None:
            ref = got
        else:
            for n in got:
                if got[n] is not None:
                    assert np.array_equal(got[n], ref[n]), (v, n)
    lat = gpu.Lattice(p, seed=8)
    upload(lat, f)
    before = lat.download()
    choices, ms = lat.autotune()
    assert all(0 <= c < 4 for c in choices)
    after = lat.download()  # autotuning does not advance the chain
    for n in before:
        if before[n] is not None:
            assert np.array_equal(before[n], after[n]), n
    assert not lat.counters().any()
