"""Statistical parity of the stochastic updates.

* KS test of single-link heatbath draws: one half-sweep from a cold pure-gauge
  lattice gives independent a0 draws with alpha = 4 beta (every staple is
  -2 beta * 1); they must follow sqrt(1 - a0^2) exp(alpha a0) (heatbath.c:30-71),
  and the vector part must point uniformly on the sphere.  FP64 uses the
  reference's algorithm, FP32 its direct-sampling variant.
* Per-kernel parity: one half-sweep of every update kernel against the oracle's
  site-by-site update with the same uniforms (FP64, 1e-11).
* Observable parity: plaquette, phi^dagger phi and the hopping term of
  independent chains of the GPU FP64 path, the GPU FP32 form and the CPU
  oracle agree within 3 sigma of binned jackknife errors (per chain, aware of
  its autocorrelation, combined over the chains), and their histograms agree
  (chi-square with counts deflated by 2 tau_int, p > 1e-3); the same for the
  multicanonical order parameter of a READONLY multicanonical run.
"""
import numpy as np
import pytest

from native import Oracle, WeightBuf, hot_fields
from stats import compare_chain_means, compare_means, histogram_pvalue, kp_a0_cdf
from su2higgs_gb300 import abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from su2higgs_gb300 import gpu as g
    g.lib()
    return g


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("beta", [2.0, 8.0])
def test_heatbath_a0_distribution(gpu, precision, beta):
    from scipy import stats as st
    p = abi.make_params("pure", L=(32, 32, 32), precision=precision, betasu2=beta)
    lat = gpu.Lattice(p, seed=int(1000 * beta) + precision)
    lat.run_halfsweep(0, 0, 0, 0, 7)
    half = p.sites() // 2
    u = lat.download()["link"][:half, 0, :]
    a0 = u[:, 0]
    ks = st.kstest(a0, kp_a0_cdf(4.0 * beta))
    assert ks.pvalue > 1e-3, ks
    r = u[:, 1:]
    rn = np.linalg.norm(r, axis=1)
    tol = 1e-12 if precision == 64 else 2e-6
    assert np.max(np.abs(rn ** 2 + a0 ** 2 - 1.0)) < tol
    z = r[:, 2] / rn
    assert st.kstest(z, "uniform", args=(-1, 2)).pvalue > 1e-3
    phi = np.arctan2(r[:, 1], r[:, 0])
    assert st.kstest(phi, "uniform", args=(-np.pi, 2 * np.pi)).pvalue > 1e-3
    assert lat.counters()[abi.C_KP_CAP] == 0
    assert lat.counters()[abi.C_ACC_SU2LINK] == half


# (gpu kind, oracle kind, sub, content, params)
KERNELS = [
    (0, 1, 1, "fund", {}),
    (0, 2, 2, "fund", dict(algorithm_su2link=abi.METROPOLIS)),
    (0, 1, 0, "adj", {}),
    (1, 3, 1, "su2u1s", {}),
    (2, 4, 0, "su2u1s", {}),
    (3, 5, 0, "su2u1s", {}),
    (2, 5, 0, "fund", dict(algorithm_su2doublet=abi.METROPOLIS)),
    (4, 6, 0, "adj", {}),
    (5, 7, 0, "adj", {}),
    (6, 8, 0, "su2u1s", {}),
    (7, 9, 0, "su2u1s", {}),
    (2, 4, 0, "higgs2", {}),
    (2, 4, 1, "higgs2", {}),
    (4, 6, 0, "fundadj", {}),
]


@pytest.mark.parametrize("gk,ok,sub,content,kw", KERNELS)
@pytest.mark.parametrize("parity", [0, 1])
def test_halfsweep_matches_oracle(gpu, gk, ok, sub, content, kw, parity):
    p = abi.make_params(content, L=(8, 6, 10), **kw)
    f = hot_fields(p, seed=17 + gk, phi_mean=0.5)
    seed, sweep, pss = 4242, 11, 5
    lat = gpu.Lattice(p, seed=seed)
    lat.upload(link=f.link, u1=f.u1, d0=f.d0, d1=f.d1, trip=f.trip, sing=f.sing)
    lat.run_halfsweep(gk, parity, sub, pss, sweep)
    o = Oracle(p)
    o.put(f)
    o.set_rng(seed, sweep)
    half = p.sites() // 2
    acc = 0
    for t in range(half):
        acc += o.lib.orc_site_update(o.h, ok, parity * half + t, sub, pss)
    got, want = lat.download(), o.get()
    for n in ("link", "u1", "d0", "d1", "trip", "sing"):
        w = getattr(want, n)
        if w is not None:
            assert np.max(np.abs(got[n] - w)) < 1e-11, n
    c = lat.counters()
    assert int(c[[1, 3, 6 + sub, 10 + sub, 13, 15, 17, 19]].sum()) == acc


def run_chains_gpu(gpu, p, fields, seed, ntherm, nmeas):
    """Independent chains in one pool (one per start configuration):
    per chain, the (plaquette, phi^2, hopping) series."""
    pool = gpu.Pool(p, arena_bytes=64 << 20, max_chains=len(fields))
    slots = []
    for k, f in enumerate(fields):
        s = pool.add(p, seed=seed + k, chain=k)
        pool.upload(s, link=f.link, d0=f.d0)
        slots.append(s)
    pool.run(ntherm)
    V = p.sites()
    rows = {s: [] for s in slots}
    for _ in range(nmeas):
        pool.run(1)
        for s, m in pool.measure().items():
            rows[s].append((m[abi.M_WILSON] / (V * p.betasu2), m[abi.M_PHI2] / V, m[abi.M_COV_PHI] / (3 * V)))
    pool.close()
    return [np.array(rows[s]) for s in slots]


def run_chain_oracle(p, f, seed, ntherm, nmeas, chain=0):
    o = Oracle(p)
    o.put(f)
    V = p.sites()
    for s in range(ntherm):
        o.set_rng(seed, s, chain)
        o.update()
    rows = []
    for s in range(nmeas):
        o.set_rng(seed, ntherm + s, chain)
        o.update()
        m = o.measure()
        rows.append((m[abi.M_WILSON] / (V * p.betasu2), m[abi.M_PHI2] / V, m[abi.M_COV_PHI] / (3 * V)))
    return np.array(rows)


def test_observables_gpu64_gpu32_oracle(gpu):
    """Config-1 couplings (beta 8, m^2 -0.1, lambda 0.002) on 8^3: the three
    implementations sample the same distribution.  Independent chains per
    implementation (GPU: 8 chains in a pool; oracle: 4), errors from the
    chains' binned jackknife errors combined."""
    p64 = abi.make_params("fund", L=(8, 8, 8))
    p32 = abi.make_params("fund", L=(8, 8, 8), precision=32)
    starts = [hot_fields(p64, seed=5 + k, phi_mean=1.0) for k in range(8)]
    n_therm = 300
    a = run_chains_gpu(gpu, p64, starts, 101, n_therm, 6000)
    b = run_chains_gpu(gpu, p32, starts, 202, n_therm, 6000)
    c = [run_chain_oracle(p64, starts[k], 303, n_therm, 3000, chain=k) for k in range(4)]
    names = ["plaquette", "phi2", "hopping"]
    for k, name in enumerate(names):
        for (x, y, tag) in ((a, c, "gpu64-oracle"), (b, c, "gpu32-oracle"), (a, b, "gpu64-gpu32")):
            z, mx, my = compare_chain_means([r[:, k] for r in x], [r[:, k] for r in y])
            assert z < 3.0, (name, tag, z, mx, my)
            pv = histogram_pvalue(np.concatenate([r[:, k] for r in x]), np.concatenate([r[:, k] for r in y]))
            assert pv > 1e-3, (name, tag, pv)


@pytest.mark.parametrize("content", ["fund", "su2u1s"])
@pytest.mark.parametrize("precision", [64, 32])
def test_multicanonical_orderparam_distribution(gpu, precision, content):
    """READONLY multicanonical run (global accept/reject after each doublet
    half-sweep, multicanonical.c:385-445 with the order parameter of
    multicanonical.c:709-751): the order-parameter distribution of the GPU
    (FP64 fields, and FP32 fields with the FP64 weight and decisions) and of
    the oracle, for SU(2) + Higgs and for SU(2) x U(1) + Higgs + singlet
    (the multicanonical workload's content)."""
    p = abi.make_params(content, L=(6, 6, 6))
    f = hot_fields(p, seed=8, phi_mean=1.0)
    # warm up to equilibrium with the oracle, then centre a tilted weight there
    o0 = Oracle(p)
    o0.put(f)
    for s in range(200):
        o0.set_rng(7, s)
        o0.update()
    f0 = o0.get()
    R0 = float(np.mean(0.5 * np.sum(f0.d0 ** 2, axis=1)))
    bins = 16
    w = WeightBuf(bins, orderparam=abi.PHISQ, mode=abi.MUCA_READONLY)
    lo, hi = R0 - 0.3, R0 + 0.3
    w.pos[1:] = np.linspace(lo, hi, bins + 1)
    w.pos[0] = lo - 1000 * (hi - lo)
    w.W[1:] = 20.0 * (w.pos[1:] - R0) ** 2
    w.W[0] = w.W[1]
    w.W[bins + 1] = w.W[bins]
    w.linearize()
    s = w.struct
    s.min, s.max, s.wrk_min, s.wrk_max = lo, hi, lo, hi
    half = p.sites() // 2
    ph = 0.5 * np.sum(f0.d0 ** 2, axis=1)
    s.param_value[0] = ph[:half].sum() / p.sites()
    s.param_value[1] = ph[half:].sum() / p.sites()
    nmeas = 3000
    lat = gpu.Lattice(abi.make_params(content, L=(6, 6, 6), precision=precision), seed=55)
    lat.upload(link=f0.link, u1=f0.u1, d0=f0.d0, sing=f0.sing)
    lat.muca_set(s)
    o = Oracle(p)
    o.put(f0)
    o.muca_set(w)
    ga, oa = [], []
    wg = WeightBuf(bins)
    for k in range(nmeas):
        lat.update_lattice(k)
        lat.muca_get(wg.struct)
        ga.append(wg.struct.param_value[0] + wg.struct.param_value[1])
        o.set_rng(66, k)
        o.update()
        wo = WeightBuf(bins)
        o.muca_get(wo)
        oa.append(wo.struct.param_value[0] + wo.struct.param_value[1])
    ga, oa = np.array(ga), np.array(oa)
    z, mg, mo = compare_means(ga, oa)
    assert z < 3.0, (z, mg, mo)
    assert histogram_pvalue(ga, oa) > 1e-3
    cg, co = lat.counters(), o.counters()
    rate_g = cg[abi.C_ACC_MUCA] / cg[abi.C_TOTAL_MUCA]
    rate_o = co[abi.C_ACC_MUCA] / co[abi.C_TOTAL_MUCA]
    assert 0.05 < rate_g < 0.999 and abs(rate_g - rate_o) < 0.05, (rate_g, rate_o)


def _starts(p, n, seed, broken=0.0, **kw):
    """Start configurations: hot (Haar links, normal scalars), or, with
    `broken`, cold links and the triplet aligned at `broken` along its first
    component (plus noise): a broken-phase start without monopoles, which a
    hot start can trap in the Higgs phase as a frozen monopole pair."""
    out = []
    for k in range(n):
        f = hot_fields(p, seed=seed + k, **kw)
        if broken and f.trip is not None:
            f.link[:] = 0.0
            f.link[..., 0] = 1.0
            f.trip[:, 0] += broken
        out.append({n_: getattr(f, n_) for n_ in ("link", "u1", "d0", "d1", "trip", "sing")})
    return out


# SU(2) + adjoint Higgs at couplings of the batched ensemble (beta in [6, 12],
# m^2_adj in [-0.3, 0.1], lambda_adj 0.005), one point on each side of the
# transition on 8^3: beta 12, m^2 -0.3 started in the broken phase (Tr Sigma^2
# ~ 23.5, no monopoles), beta 8, m^2 0.1 in the symmetric phase (Tr Sigma^2 ~
# 0.3).  Observables of measure.c:110-174: plaquette, Tr Sigma^2,
# hopping_Sigma, |magnetic charge| density.
ADJ_POINTS = {
    "broken": dict(betasu2=12.0, msq_triplet=-0.3, b4=0.005, broken=6.8, trip_sigma=0.1),
    "symmetric": dict(betasu2=8.0, msq_triplet=0.1, b4=0.005, broken=0.0, trip_sigma=0.3),
}


@pytest.mark.parametrize("point", sorted(ADJ_POINTS))
def test_adjoint_fp32_observables_match_oracle(gpu, point):
    """The headline form's chains -- FP32 fields in a pool swept by the
    persistent work-list kernel -- against FP64 GPU pool chains and the FP64
    oracle from the same starts: every observable within 3 sigma of the
    binned jackknife errors and equal histograms (heatbath.c:21-27,107-120,
    overrelax.c:137-236, metropolis.c:113-143)."""
    import chains
    kw = dict(ADJ_POINTS[point])
    broken = kw.pop("broken")
    trip_sigma = kw.pop("trip_sigma")
    L = (8, 8, 8)
    p32 = abi.make_params("adj", L=L, precision=32, **kw)
    p64 = abi.make_params("adj", L=L, precision=64, **kw)
    starts = _starts(p64, 8, 900, broken=broken, trip_sigma=trip_sigma)
    n_therm, n_gpu, n_orc = 400, 4000, 2000
    orc = chains.oracle_chains("adj", L, kw, starts[:4], 303, n_therm, n_orc)
    g32 = chains.pool_chains(gpu, p32, starts, 101, n_therm, n_gpu, persistent=True)
    g64 = chains.pool_chains(gpu, p64, starts, 202, n_therm, n_gpu)
    names = chains.CONTENT_OBSERVABLES["adj"]
    rows, fails = chains.compare(names, {"fp32": g32, "fp64": g64, "oracle": orc})
    print("\n" + chains.format_rows(f"adjoint 8^3 {point} {kw}", rows))
    assert not fails, fails


def test_su2u1s_fp32_observables_match_oracle(gpu):
    """SU(2) x U(1) + doublet + singlet (the multicanonical workload's
    content, beta_G 8, beta_U1 24) without multicanonical acceptance: FP32
    GPU chains against FP64 GPU chains and the oracle."""
    import chains
    L = (8, 8, 8)
    p32 = abi.make_params("su2u1s", L=L, precision=32)
    p64 = abi.make_params("su2u1s", L=L, precision=64)
    starts = _starts(p64, 8, 950, phi_mean=1.0)
    n_therm, n_gpu, n_orc = 300, 4000, 2000
    orc = chains.oracle_chains("su2u1s", L, {}, starts[:4], 313, n_therm, n_orc)
    g32 = chains.pool_chains(gpu, p32, starts, 111, n_therm, n_gpu, persistent=True)
    g64 = chains.pool_chains(gpu, p64, starts, 212, n_therm, n_gpu)
    names = chains.CONTENT_OBSERVABLES["su2u1s"]
    rows, fails = chains.compare(names, {"fp32": g32, "fp64": g64, "oracle": orc})
    print("\n" + chains.format_rows("su2u1s 8^3", rows))
    assert not fails, fails


# the FP32 form against the FP64 path at high statistics: 64 independent
# pool chains of 8^3 each, 20000 measured sweeps per chain, the recipe of the
# workloads (link heatbath, 4 overrelaxation + 1 Metropolis sweeps of the
# scalars)
HIGH_STAT_CASES = {
    "fund": ({}, dict(phi_mean=1.0)),
    "adj": (dict(betasu2=8.0, msq_triplet=0.1, b4=0.005), dict(trip_sigma=0.3)),
    "su2u1s": ({}, dict(phi_mean=1.0)),
}


@pytest.mark.parametrize("content", sorted(HIGH_STAT_CASES))
def test_fp32_against_fp64_high_statistics(gpu, content):
    """Every observable of the FP32 form equals the FP64 path's within 3
    sigma at errors of ~1e-5 (plaquette) to ~1e-4 (scalar observables)
    relative: the FP32 arithmetic (24-bit uniforms, direct sphere sampling,
    approximate division and square root, links re-normalised at every write)
    leaves no bias at that level."""
    import chains
    kw, skw = HIGH_STAT_CASES[content]
    L = (8, 8, 8)
    p32 = abi.make_params(content, L=L, precision=32, **kw)
    p64 = abi.make_params(content, L=L, precision=64, **kw)
    starts = _starts(p64, 64, 1900, **skw)
    g32 = chains.pool_chains(gpu, p32, starts, 1101, 300, 20000)
    g64 = chains.pool_chains(gpu, p64, starts, 1202, 300, 20000)
    names = chains.CONTENT_OBSERVABLES[content]
    rows, fails = chains.compare(names, {"fp32": g32, "fp64": g64})
    print("\n" + chains.format_rows(f"{content} 8^3, 64 chains x 20000 sweeps {kw}", rows))
    assert not fails, fails
