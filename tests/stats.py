"""Statistics used by the statistical parity tests: integrated
autocorrelation time, binned jackknife errors, a histogram comparison that
accounts for autocorrelation, and the Kennedy-Pendleton a0 distribution."""
import numpy as np


def tau_int(x, window_c=6.0):
    """Integrated autocorrelation time with Sokal's automatic window."""
    x = np.asarray(x, dtype=np.float64)
    n = len(x)
    x = x - x.mean()
    var = np.dot(x, x) / n
    if var == 0:
        return 0.5
    f = np.fft.rfft(x, 2 * n)
    acf = np.fft.irfft(f * np.conj(f))[:n] / (var * np.arange(n, 0, -1))
    tau = 0.5
    for w in range(1, n // 2):
        tau += acf[w]
        if w >= window_c * tau:
            break
    return max(tau, 0.5)


def jackknife_mean(x, nbins=None):
    """Mean and jackknife error with bins of at least 4 tau_int."""
    x = np.asarray(x, dtype=np.float64)
    t = tau_int(x)
    size = max(1, int(np.ceil(4 * t)))
    nb = nbins or max(8, len(x) // size)
    nb = min(nb, len(x))
    m = len(x) // nb * nb
    bins = x[:m].reshape(nb, -1).mean(axis=1)
    tot = bins.sum()
    jk = (tot - bins) / (nb - 1)
    err = np.sqrt((nb - 1) / nb * np.sum((jk - jk.mean()) ** 2))
    return x[:m].mean(), err, t


def compare_means(a, b):
    """|mean(a) - mean(b)| in units of the combined jackknife error."""
    ma, ea, _ = jackknife_mean(a)
    mb, eb, _ = jackknife_mean(b)
    return abs(ma - mb) / np.sqrt(ea ** 2 + eb ** 2 + 1e-300), (ma, ea), (mb, eb)


def histogram_edges(x, nbins):
    """Bin edges at the quantiles of x, each moved to the midpoint between the
    two neighbouring distinct values (x rounded to 1e-5 of its range): an
    observable that takes discrete values (the monopole density, a count)
    then never has a level on an edge, where rounding differences of 1e-16
    (or 1e-7 with FP32 fields) between two implementations would send the
    same level to different bins.  For continuous data the move is below the
    spacing of the samples."""
    x = np.asarray(x, dtype=np.float64)
    lo, hi = float(np.min(x)), float(np.max(x))
    scale = (hi - lo) or 1.0
    levels = np.unique(np.round((x - lo) / scale, 5)) * scale + lo
    q = np.quantile(x, np.linspace(0, 1, nbins + 1))[1:-1]
    k = np.clip(np.searchsorted(levels, q), 1, max(1, len(levels) - 1))
    inner = np.unique(0.5 * (levels[k - 1] + levels[np.minimum(k, len(levels) - 1)]))
    inner = inner[(inner > lo) & (inner < hi)]
    return np.concatenate([[lo - 1e-12 * scale], inner, [hi + 1e-12 * scale]])


def histogram_pvalue(a, b, nbins=10):
    """Two-sample chi-square test of equal histograms with counts deflated by
    2 tau_int (the effective number of independent samples)."""
    from scipy import stats as st
    a = np.asarray(a)
    b = np.asarray(b)
    edges = histogram_edges(np.concatenate([a, b]), nbins)
    ha, _ = np.histogram(a, edges)
    hb, _ = np.histogram(b, edges)
    ta, tb = tau_int(a), tau_int(b)
    ha = ha / (2 * ta)
    hb = hb / (2 * tb)
    na, nb = ha.sum(), hb.sum()
    ka, kb = np.sqrt(nb / na), np.sqrt(na / nb)
    mask = (ha + hb) > 0
    chi2 = np.sum((ka * ha[mask] - kb * hb[mask]) ** 2 / (ha[mask] + hb[mask]))
    dof = mask.sum() - 1
    return float(st.chi2.sf(chi2, dof))


def kp_a0_cdf(alpha):
    """CDF of a0 with density sqrt(1 - a0^2) exp(alpha a0) on [-1, 1]
    (the distribution the Kennedy-Pendleton heatbath samples, heatbath.c:30-71),
    by numerical integration in y = 1 - a0."""
    y = np.concatenate([np.geomspace(1e-12, 2.0, 200001)])
    y = np.concatenate([[0.0], y])
    dens = np.sqrt(np.clip(y * (2 - y), 0, None)) * np.exp(-alpha * y)
    cum = np.concatenate([[0.0], np.cumsum(0.5 * (dens[1:] + dens[:-1]) * np.diff(y))])
    cum /= cum[-1]
    # a0 = 1 - y: P(A0 <= a) = P(Y >= 1 - a) = 1 - F_Y(1 - a)

    def cdf(a):
        a = np.asarray(a, dtype=np.float64)
        return 1.0 - np.interp(1.0 - a, y, cum)
    return cdf


def chains_mean(chains):
    """Mean over independent chains and its error: the chains' binned
    jackknife errors (each aware of its own autocorrelation) combined, or,
    with 8 chains or more, the spread of the chain means if that is larger.
    The spread needs no autocorrelation estimate: repeated 64-chain runs of
    slow observables (the adjoint Tr Sigma^2 and hopping term at 8^3) with
    other seeds scattered about twice as far as the combined jackknife errors
    said, so the per-chain windows can understate the error."""
    ms, es = [], []
    for x in chains:
        m, e, _ = jackknife_mean(x)
        ms.append(m)
        es.append(e)
    n = len(ms)
    err = float(np.sqrt(np.sum(np.square(es))) / n)
    if n >= 8:
        err = max(err, float(np.std(ms, ddof=1) / np.sqrt(n)))
    return float(np.mean(ms)), err


def compare_chain_means(a_chains, b_chains):
    """|mean(a) - mean(b)| in units of the combined error, for two sets of
    independent chains."""
    ma, ea = chains_mean(a_chains)
    mb, eb = chains_mean(b_chains)
    return abs(ma - mb) / np.sqrt(ea ** 2 + eb ** 2 + 1e-300), (ma, ea), (mb, eb)
