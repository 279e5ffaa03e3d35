"""Independent Monte Carlo chains for the statistical parity tests: GPU pool
chains (FP32 or FP64, optionally the persistent sweep) and oracle chains run
in worker processes, with the observables the reference's measure() rows
carry (measure.c:110-233) as volume averages.

The oracle workers are started with the `spawn` method, so that no child
inherits a CUDA context; they rebuild their lattice from plain arguments
(content name, sides, couplings, start fields as numpy arrays).
"""
import multiprocessing as mp

import numpy as np

from stats import compare_chain_means, histogram_pvalue
from su2higgs_gb300 import abi

# observable name -> (measure() column, divisor: "V", "3V", "betaV")
OBSERVABLES = {
    "plaquette": (abi.M_WILSON, "betaV"),  # beta-normalised Wilson action per site
    "u1_plaquette": (abi.M_U1WILSON, "V"),
    "phi2": (abi.M_PHI2, "V"),
    "hopping_phi": (abi.M_COV_PHI, "3V"),
    "sigma2": (abi.M_SIGMA2, "V"),
    "hopping_sigma": (abi.M_HOP_SIGMA, "3V"),
    "magcharge_abs": (abi.M_MAGCHARGE_ABS, "V"),
    "singlet": (abi.M_S1, "V"),
    "singlet2": (abi.M_S2, "V"),
}

CONTENT_OBSERVABLES = {
    "fund": ["plaquette", "phi2", "hopping_phi"],
    "adj": ["plaquette", "sigma2", "hopping_sigma", "magcharge_abs"],
    "su2u1s": ["plaquette", "u1_plaquette", "phi2", "hopping_phi", "singlet", "singlet2"],
}


def observables(names, m, V, beta):
    out = []
    for n in names:
        col, div = OBSERVABLES[n]
        d = {"V": V, "3V": 3 * V, "betaV": beta * V}[div]
        out.append(m[col] / d)
    return out


def pool_chains(gpu, p, starts, seed, ntherm, nmeas, persistent=None):
    """One pool chain per start configuration (seed + k, chain id k): per
    chain the series of the content's observables, one row per sweep."""
    names = CONTENT_OBSERVABLES[_content_name(p)]
    pool = gpu.Pool(p, arena_bytes=64 << 20, max_chains=len(starts))
    pool.persistent = persistent
    slots = []
    for k, f in enumerate(starts):
        s = pool.add(p, seed=seed + k, chain=k)
        pool.upload(s, **{n: f[n] for n in f if f[n] is not None})
        slots.append(s)
    pool.run(ntherm)
    V = p.sites()
    rows = {s: [] for s in slots}
    for _ in range(nmeas):
        pool.run(1)
        for s, m in pool.measure().items():
            rows[s].append(observables(names, m, V, p.betasu2))
    pool.close()
    return [np.array(rows[s]) for s in slots]


def _content_name(p):
    for name, bits in abi.CONTENTS.items():
        if bits == p.content:
            return name
    raise KeyError(p.content)


def _oracle_chain(args):
    import sys
    import os
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from native import Fields, Oracle
    content, L, kw, start, seed, chain, ntherm, nmeas = args
    p = abi.make_params(content, L=L, **kw)
    o = Oracle(p)
    o.put(Fields(p, **start))
    names = CONTENT_OBSERVABLES[content]
    V = p.sites()
    for s in range(ntherm):
        o.set_rng(seed, s, chain)
        o.update()
    rows = []
    for s in range(nmeas):
        o.set_rng(seed, ntherm + s, chain)
        o.update()
        rows.append(observables(names, o.measure(), V, p.betasu2))
    return np.array(rows)


def oracle_chains(content, L, kw, starts, seed, ntherm, nmeas, workers=None):
    """Oracle (FP64 CPU restatement) chains, one per start, in parallel worker
    processes (spawned)."""
    jobs = [(content, tuple(L), dict(kw), {n: f[n] for n in f if f[n] is not None}, seed, k, ntherm, nmeas)
            for k, f in enumerate(starts)]
    ctx = mp.get_context("spawn")
    with ctx.Pool(workers or min(len(jobs), max(1, mp.cpu_count() - 1))) as pool:
        return pool.map(_oracle_chain, jobs, chunksize=1)


# an observable whose every sample lies within ZERO of 0 in both sets being
# compared is zero up to rounding in both (the monopole density of the
# broken phase: ~1e-16 with FP64 fields, ~1e-8 with FP32 ones)
ZERO = 1e-5


def compare(names, sets, z_max=3.0, p_min=1e-3):
    """Pairwise comparison of chain sets {label: [chain arrays]}: per
    observable and pair, |difference| in units of the combined jackknife
    error (z) and the histogram p-value.  Returns (table rows, failures)."""
    labels = list(sets)
    rows, fails = [], []
    for k, name in enumerate(names):
        for i in range(len(labels)):
            for j in range(i + 1, len(labels)):
                a, b = labels[i], labels[j]
                z, (ma, ea), (mb, eb) = compare_chain_means([x[:, k] for x in sets[a]], [x[:, k] for x in sets[b]])
                xa = np.concatenate([x[:, k] for x in sets[a]])
                xb = np.concatenate([x[:, k] for x in sets[b]])
                if max(np.max(np.abs(xa)), np.max(np.abs(xb))) < ZERO:
                    z, pv = 0.0, 1.0  # zero up to rounding in both
                else:
                    pv = histogram_pvalue(xa, xb)
                rows.append((name, a, b, ma, ea, mb, eb, ma - mb, float(np.hypot(ea, eb)), z, pv))
                if z >= z_max or pv <= p_min:
                    fails.append((name, a, b, z, pv, (ma, ea), (mb, eb)))
    return rows, fails


def format_rows(title, rows):
    out = [title]
    for name, a, b, ma, ea, mb, eb, d, ed, z, pv in rows:
        out.append(f"  {name:14s} {a}-{b}: {ma:.6g}+-{ea:.2g} vs {mb:.6g}+-{eb:.2g}  diff {d:+.3g}+-{ed:.2g}"
                   f"  z {z:.2f}  hist p {pv:.3g}")
    return "\n".join(out)
