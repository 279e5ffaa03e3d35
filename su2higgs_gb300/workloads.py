"""Seeded synthetic inputs of the named workloads: hot-start fields and the
batched ensemble of independent chains.

The reference's runs start from a hot or cold lattice made by its own
initialisation (init.c:18-60) and measure on configurations it generated; no
dataset is involved.  These generators give the same kind of input: Haar-random
SU(2) links (four normals normalised), scalar components drawn from normal
distributions, and coupling sets drawn within the ranges of the workload.
"""
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
