"""The oracle (oracle/src, CPU restatement) against the golden fixtures made by
the reference itself.  Pins the oracle wherever the reference is absent."""
import numpy as np
import pytest

from golden_io import fields_of, load, measure_close, names, params_of, weight_of
from native import Oracle, ref_sums_to_layout, rel_err
from su2higgs_gb300 import abi

# deterministic arithmetic: the oracle and the reference differ by rounding only
RTOL_DET = 1e-12
# after several stochastic sweeps rounding differences grow chaotically but
# decisions agree; the fields must still agree far inside this bound
ATOL_FIELDS_1 = 1e-11
ATOL_FIELDS_3 = 1e-9


@pytest.mark.parametrize("name", names("layout_"))
def test_layout_tables_bit_exact(name):
    d = load(name)
    L = tuple(int(x) for x in d["L"])
    o = Oracle(abi.make_params("pure", L=L))
    nx, pv, co, par = o.tables()
    assert np.array_equal(nx, d["next"])
    assert np.array_equal(pv, d["prev"])
    assert np.array_equal(co, d["coords"])
    assert np.array_equal(par, d["parity"])


@pytest.mark.parametrize("name", names("sites_"))
def test_site_kernels(name):
    import ctypes
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    d = load(name)
    p = params_of(d)
    o = Oracle(p)
    o.put(fields_of(d, p, "in_"))
    lib, h, V, D = o.lib, o.h, o.V, p.dim
    st = np.zeros((V, D, 4))
    ws = np.zeros((V, D, 4))
    for i in range(V):
        for mu in range(D):
            lib.orc_link_staple(h, i, mu, P(st[i, mu]))
            lib.orc_wilson_staple(h, i, mu, P(ws[i, mu]))
    assert rel_err(st, d["link_staple"], 1e-3) < RTOL_DET
    assert rel_err(ws, d["wilson_staple"], 1e-3) < RTOL_DET
    la = np.array([[lib.orc_localact_su2link(h, i, mu) for mu in range(D)] for i in range(V)])
    assert rel_err(la, d["localact_su2link"]) < RTOL_DET
    assert rel_err([lib.orc_action_local(h, i) for i in range(V)], d["action_local"]) < RTOL_DET
    assert rel_err([lib.orc_local_su2wilson(h, i) for i in range(V)], d["local_su2wilson"]) < RTOL_DET
    if "localact_u1link" in d:
        lu = [[lib.orc_localact_u1link(h, i, mu) for mu in range(D)] for i in range(V)]
        assert rel_err(lu, d["localact_u1link"]) < RTOL_DET
    if "staple_doublet" in d:
        sd = np.zeros((V, 4))
        for i in range(V):
            lib.orc_staple_doublet(h, i, 0, P(sd[i]))
        assert rel_err(sd, d["staple_doublet"], 1e-3) < RTOL_DET
        assert rel_err([lib.orc_localact_doublet(h, i, 0) for i in range(V)], d["localact_doublet"]) < RTOL_DET
    if "localact_triplet" in d:
        assert rel_err([lib.orc_localact_triplet(h, i) for i in range(V)], d["localact_triplet"]) < RTOL_DET
        ap = [[lib.orc_alpha_proj(h, i, a, b) for (a, b) in ((0, 1), (0, 2), (1, 2))] for i in range(V)]
        assert rel_err(ap, d["alpha_proj"], 1e-6) < RTOL_DET
        mc = np.array([lib.orc_magcharge_cube(h, i) for i in range(V)])
        assert np.max(np.abs(mc - d["magcharge_cube"])) < 1e-10
    if "localact_singlet" in d:
        assert rel_err([lib.orc_localact_singlet(h, i) for i in range(V)], d["localact_singlet"]) < RTOL_DET
    for key, kind, sub, n in (("or_doublet", 4, 0, 4), ("or_doublet1", 4, 1, 4), ("or_triplet", 6, 0, 3),
                              ("or_singlet", 8, 0, 1)):
        if key in d:
            got = np.zeros((V, n))
            for i in range(V):
                assert lib.orc_or_proposal(h, kind, i, sub, P(got[i])) == n
            assert rel_err(got if n > 1 else got[:, 0], d[key], 1e-3) < RTOL_DET, key
    ok, k, a, b = measure_close(o.measure(), d["measure"], RTOL_DET)
    assert ok, (k, a, b)


def test_layout_table_digests():
    """The closed-form layout of the larger sides (up to 128^3) against the
    SHA-256 of the reference's own layout() tables."""
    from native import layout_digest
    d = load("tables_sha256.npz")
    for L, digest in zip(d["L"], d["sha256"]):
        o = Oracle(abi.make_params("pure", L=tuple(int(x) for x in L)))
        assert layout_digest(*o.tables()) == str(digest), tuple(L)


@pytest.mark.parametrize("name", names("sweep_"))
def test_sweeps(name):
    d = load(name)
    p = params_of(d)
    o = Oracle(p)
    o.put(fields_of(d, p, "in_"))
    seed, s0 = int(d["seed"]), int(d["first_sweep"])
    o.set_rng(seed, s0)
    assert o.update() == int(d["npasses"])
    out1 = fields_of(d, p, "out1_")
    for k, v in o.get().max_abs_diff(out1).items():
        assert v < ATOL_FIELDS_1, (k, v)
    assert np.array_equal(o.counters()[:22], d["counters1"][:22])
    for s in (s0 + 1, s0 + 2):
        o.set_rng(seed, s)
        o.update()
    out3 = fields_of(d, p, "out3_")
    for k, v in o.get().max_abs_diff(out3).items():
        assert v < ATOL_FIELDS_3, (k, v)
    assert np.array_equal(o.counters()[:22], d["counters3"][:22])
    ok, k, a, b = measure_close(o.measure(), d["measure3"], 1e-8)
    assert ok, (k, a, b)


@pytest.mark.parametrize("name", names("muca_"))
def test_muca(name):
    d = load(name)
    p = params_of(d)
    o = Oracle(p)
    o.put(fields_of(d, p, "in_"))
    w = weight_of(d, "w0_")
    o.muca_set(w)
    seed = int(d["seed"])
    for s in range(int(d["nsweeps"])):
        o.set_rng(seed, 100 + s)
        o.update()
    out = fields_of(d, p, "out_")
    for k, v in o.get().max_abs_diff(out).items():
        assert v < ATOL_FIELDS_3, (k, v)
    assert np.array_equal(o.counters()[:22], d["counters"][:22])
    w1 = weight_of(d, "w1_")
    o.muca_get(w)
    assert np.array_equal(w.hits, w1.hits)
    assert rel_err(w.W, w1.W, 1e-9) < 1e-9
    assert w.struct.last_max == w1.struct.last_max
    assert w.struct.muca_count == w1.struct.muca_count
    assert abs(w.struct.delta - w1.struct.delta) < 1e-15
    assert rel_err(list(w.struct.param_value), list(w1.struct.param_value)) < 1e-9
    if w.struct.mode == abi.MUCA_SLOW:  # update_weight_slow's accumulators
        assert np.array_equal(w.gsum, w1.gsum) and np.array_equal(w.nsum, w1.nsum)
        assert rel_err(w.hgram, w1.hgram, 1e-9) < 1e-9


@pytest.mark.parametrize("name", names("flow_"))
def test_flow(name):
    d = load(name)
    p = params_of(d)
    o = Oracle(p)
    o.put(fields_of(d, p, "in_"))
    rows = o.grad_flow(float(d["t_max"]), float(d["dt"]), int(d["meas_interval"]))
    ref_rows = d["rows_raw"]
    assert rows.shape[0] == ref_rows.shape[0]
    for r_o, r_r in zip(rows, ref_rows):
        ok, k, a, b = measure_close(r_o[1:], ref_sums_to_layout(p, r_r), 1e-11)
        assert ok, (k, a, b)
    o.lib.orc_flow_step(o.h, float(d["dt"]))
    step = fields_of(d, p, "step_")
    for k, v in o.get().max_abs_diff(step).items():
        assert v < 1e-13, (k, v)


@pytest.mark.parametrize("name", names("correl_"))
def test_correlators(name):
    """measure_correlators (correlation.c:350-398) along the longest
    direction, and on every blocking level the smeared, blocked links and
    triplet (su2u1.c:752-905, blocking.c:296-374) in the blocked lattice's
    storage order and the correlators measured there; 1e-12 relative to the
    largest value of a column (the values are sums of products of plane sums
    in another order), fields 1e-13."""
    d = load(name)
    p = params_of(d)
    o = Oracle(p)
    o.put(fields_of(d, p, "in_"))
    ld = int(d["dir"])
    assert o.longest_dir() == ld
    corr_close(o.correlators(ld), d["corr0"])
    bd = [int(k != ld) for k in range(3)]
    cur = o
    for k in range(1, int(d["levels"]) + 1):
        cur = cur.block(bd)
        assert list(cur.p.L[:3]) == list(d[f"b{k}_L"])
        _, _, co, _ = cur.tables()
        assert np.array_equal(co, d[f"b{k}_coords"])
        got = cur.get()
        assert np.max(np.abs(got.link - d[f"b{k}_link"])) < 1e-13
        assert np.max(np.abs(got.trip - d[f"b{k}_trip"])) < 1e-13
        corr_close(cur.correlators(ld), d[f"b{k}_corr"])


def corr_close(got, want, rtol=1e-12):
    assert got.shape == want.shape
    # a photon column is scaled by the larger of its re/im pair: an imaginary
    # part that vanishes identically (a real phase) is rounding noise
    col = np.max(np.abs(want), axis=0)
    pair = np.array([c if c < 2 else c ^ 1 for c in range(want.shape[1])])
    scale = np.maximum(col, col[pair]) + 1e-300
    assert np.all(np.abs(got - want) <= rtol * scale), np.max(np.abs(got - want) / scale, axis=0)
