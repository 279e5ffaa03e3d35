"""Seeded synthetic inputs of the named workloads: hot-start fields and the
batched ensemble of independent chains.

The reference's runs start from a hot or cold lattice made by its own
initialisation (init.c:18-60) and measure on configurations it generated; no
dataset is involved.  These generators give the same kind of input: Haar-random
SU(2) links (four normals normalised), scalar components drawn from normal
distributions, and coupling sets drawn within the ranges of the workload.
"""
import ctypes

import numpy as np

from . import abi

# batched ensemble: independent SU(2) + adjoint Higgs chains
ENSEMBLE_SIDES = (8, 12, 16, 24, 32, 48)
ENSEMBLE_BETA = (6.0, 12.0)
ENSEMBLE_MSQ_ADJ = (-0.3, 0.1)
ENSEMBLE_LAMBDA_ADJ = 0.005


def hot_fields(p, seed, phi_sigma=0.1, trip_sigma=0.1, sing_sigma=0.1, u1_sigma=0.5):
    """FP64 host fields in the reference's layout order: links (V, 3, 4)
    Haar-random, doublets (V, 4), triplet (V, 3), singlet (V,), U(1) angles
    (V, 3), each present only where the content has the field."""
    rng = np.random.default_rng(seed)
    V = p.sites()
    link = rng.normal(size=(V, 3, 4))
    link /= np.linalg.norm(link, axis=2, keepdims=True)
    out = {"link": link}
    if p.content & abi.U1:
        out["u1"] = rng.normal(scale=u1_sigma, size=(V, 3))
    nh = p.nhiggs()
    if nh > 0:
        out["d0"] = rng.normal(scale=phi_sigma, size=(V, 4))
    if nh > 1:
        out["d1"] = rng.normal(scale=phi_sigma, size=(V, 4))
    if p.content & abi.TRIPLET:
        out["trip"] = rng.normal(scale=trip_sigma, size=(V, 3))
    if p.content & abi.SINGLET:
        out["sing"] = rng.normal(scale=sing_sigma, size=(V,))
    return out


def batched_ensemble(nchains=384, seed=20261203, precision=32):
    """`nchains` SU(2) + adjoint Higgs chains: side L uniform over
    ENSEMBLE_SIDES, beta uniform in ENSEMBLE_BETA, m^2_adj scanning
    ENSEMBLE_MSQ_ADJ across the chains, lambda_adj (b4) = 0.005.
    Returns [(params, seed, chain id)]."""
    rng = np.random.default_rng(seed)
    sides = rng.choice(ENSEMBLE_SIDES, size=nchains)
    betas = rng.uniform(*ENSEMBLE_BETA, size=nchains)
    msq = np.linspace(*ENSEMBLE_MSQ_ADJ, nchains)
    out = []
    for k in range(nchains):
        L = int(sides[k])
        p = abi.make_params("adj", L=(L, L, L), precision=precision, betasu2=float(betas[k]),
                            msq_triplet=float(msq[k]), b4=ENSEMBLE_LAMBDA_ADJ)
        out.append((p, seed + 7919 * k, k))
    return out


# multicanonical SU(2) x U(1) + singlet workload: 96^3, beta_G = 8,
# beta_U1 = 24, a seeded piecewise-linear weight over the phi^2 volume
# average on 256 bins spanning [0, 3], one global check per Higgs sweep
MUCA_L = 96
MUCA_BINS = 256
MUCA_RANGE = (0.0, 3.0)


class PiecewiseWeight:
    """A read-only multicanonical weight (su2gpu_weight) whose arrays live in
    numpy: `bins` bins over [lo, hi), the weight at the bin starts W, and the
    virtual bins below and above set as load_weight does
    (multicanonical.c:258-264), then linearised (multicanonical.c:337-346)."""

    def __init__(self, W, lo, hi, orderparam=abi.PHISQ, checks_per_sweep=1):
        bins = len(W) - 1
        n = bins + 2
        self.pos = np.zeros(n)
        self.W = np.zeros(n)
        self.slope = np.zeros(n)
        self.b = np.zeros(n)
        self.hits = np.zeros(n, np.int32)
        self.gsum = np.zeros(n, np.int64)
        self.nsum = np.zeros(n, np.int64)
        self.hgram = np.zeros(n)
        self.pos[1:] = lo + (hi - lo) * np.arange(bins + 1) / bins
        self.pos[0] = lo - 1000.0 * (hi - lo)
        self.W[1:] = W
        self.W[0] = self.W[1]
        self.W[bins + 1] = self.W[bins]
        self.slope[1:bins + 1] = (self.W[2:] - self.W[1:bins + 1]) / (self.pos[2:] - self.pos[1:bins + 1])
        self.b[0], self.b[bins + 1] = self.W[0], self.W[bins + 1]
        self.b[1:bins + 1] = self.W[1:bins + 1] - self.slope[1:bins + 1] * self.pos[1:bins + 1]
        s = abi.Weight()
        s.bins, s.orderparam, s.mode, s.checks_per_sweep = bins, orderparam, abi.MUCA_READONLY, checks_per_sweep
        s.do_acceptance, s.update_interval = 1, 100
        s.min, s.max, s.wrk_min, s.wrk_max, s.delta = lo, hi, lo, hi, 0.3
        D, I32, I64 = (ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int32),
                       ctypes.POINTER(ctypes.c_int64))
        s.pos, s.W = self.pos.ctypes.data_as(D), self.W.ctypes.data_as(D)
        s.slope, s.b = self.slope.ctypes.data_as(D), self.b.ctypes.data_as(D)
        s.hits = self.hits.ctypes.data_as(I32)
        s.gsum, s.nsum = self.gsum.ctypes.data_as(I64), self.nsum.ctypes.data_as(I64)
        s.hgram = self.hgram.ctypes.data_as(D)
        self.struct = s


def muca_weight(seed=20261203, bins=MUCA_BINS, lo=MUCA_RANGE[0], hi=MUCA_RANGE[1]):
    """The workload's seeded piecewise-linear weight: a linear slope plus a
    seeded random walk, sampled at the bin starts."""
    rng = np.random.default_rng(seed)
    x = lo + (hi - lo) * np.arange(bins + 1) / bins
    W = 40.0 * x + np.cumsum(rng.normal(scale=0.3, size=bins + 1))
    return PiecewiseWeight(W, lo, hi)


def muca_params(precision=32):
    return abi.make_params("su2u1s", L=(MUCA_L,) * 3, precision=precision, betasu2=8.0, betau1=24.0)
