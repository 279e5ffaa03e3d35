"""The statistics helpers of the statistical parity tests (no GPU): the
autocorrelation time, the binned jackknife and the error of a mean over
many independent chains."""
import numpy as np

from stats import chains_mean, compare_chain_means, jackknife_mean, tau_int


def ar1(rng, n, a):
    e = rng.normal(size=n)
    x = np.empty(n)
    x[0] = e[0] / np.sqrt(1 - a * a)
    for i in range(1, n):
        x[i] = a * x[i - 1] + e[i]
    return x


def test_tau_int_of_an_ar1_chain():
    # tau_int = (1 + a) / (2 (1 - a)) for an AR(1) process
    rng = np.random.default_rng(1)
    a = 0.8
    t = tau_int(ar1(rng, 200000, a))
    assert abs(t - (1 + a) / (2 * (1 - a))) < 0.5


def test_jackknife_error_of_independent_samples():
    rng = np.random.default_rng(2)
    x = rng.normal(size=40000)
    m, e, t = jackknife_mean(x)
    assert abs(e - 1 / np.sqrt(len(x))) < 0.15 / np.sqrt(len(x))
    assert t < 1.0


def test_chains_mean_is_at_least_the_spread_of_the_chain_means():
    # chains whose means scatter more than their own windows say: a slow
    # mode (an offset per chain) under fast noise
    rng = np.random.default_rng(3)
    chains = [rng.normal(size=2000) * 0.1 + rng.normal() * 0.05 for _ in range(64)]
    m, e = chains_mean(chains)
    spread = np.std([c.mean() for c in chains], ddof=1) / 8.0
    assert e >= spread * (1 - 1e-12)
    jk = np.sqrt(sum(jackknife_mean(c)[1] ** 2 for c in chains)) / 64
    assert e > 2 * jk  # the windows alone would understate it
    # few chains: the combined jackknife error alone
    m4, e4 = chains_mean(chains[:4])
    jk4 = np.sqrt(sum(jackknife_mean(c)[1] ** 2 for c in chains[:4])) / 4
    assert abs(e4 - jk4) < 1e-15


def test_compare_chain_means_z_of_equal_sets_is_small():
    rng = np.random.default_rng(4)
    a = [rng.normal(size=3000) for _ in range(16)]
    b = [rng.normal(size=3000) for _ in range(16)]
    z, (ma, ea), (mb, eb) = compare_chain_means(a, b)
    assert z < 4 and ea > 0 and eb > 0
