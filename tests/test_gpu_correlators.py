"""Correlators and blocking on the GPU (su2gpu_measure_correlators,
su2gpu_measure_blocked_correlators, su2gpu_blocked_fields) against the
reference's own values (tests/golden/correl_*.npz, made by its correlator /
blocking build through the harness) and against the oracle on larger
lattices.  Tolerances: correlators 1e-12 of the largest value of each column
(of the re/im pair for the photon columns) in FP64 -- the plane sums are
added in another order, and the phases come from sincospi where the
reference calls sin/cos of 2 pi p.x -- and 2e-5 in the FP32 form; blocked
fields 1e-13 (FP64)."""
import numpy as np
import pytest

from golden_io import fields_of, load, names, params_of
from native import Oracle, hot_fields
from su2higgs_gb300 import abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from su2higgs_gb300 import gpu as g
    g.lib()
    return g


def corr_close(got, want, rtol):
    assert got.shape == want.shape, (got.shape, want.shape)
    # a photon column is scaled by the larger of its re/im pair: an imaginary
    # part that vanishes identically (a real phase) is rounding noise
    col = np.max(np.abs(want), axis=0)
    pair = np.array([c if c < 2 else c ^ 1 for c in range(want.shape[1])])
    scale = np.maximum(col, col[pair]) + 1e-300
    err = np.max(np.abs(got - want) / scale, axis=0)
    assert np.all(err <= rtol), err


def lattice_of(gpu, d, precision):
    p64 = params_of(d)
    p = abi.make_params(p64.content, L=tuple(p64.L[:3]), precision=precision)
    for name, _ in abi.Params._fields_:
        if name not in ("L", "dim", "precision", "content"):
            setattr(p, name, getattr(p64, name))
    f = fields_of(d, p64, "in_")
    lat = gpu.Lattice(p, seed=1)
    lat.upload(link=f.link, u1=f.u1, d0=f.d0, d1=f.d1, trip=f.trip, sing=f.sing)
    return lat


def lex_order(coords, L):
    """storage index -> lexicographic index of the blocked lattice"""
    return coords[:, 0] + L[0] * (coords[:, 1] + L[1] * coords[:, 2])


@pytest.mark.parametrize("precision,rtol", [(64, 1e-12), (32, 2e-5)])
@pytest.mark.parametrize("name", names("correl_"))
def test_correlators_match_reference(gpu, name, precision, rtol):
    d = load(name)
    lat = lattice_of(gpu, d, precision)
    ld = int(d["dir"])
    assert lat.longest_dir() == ld
    corr_close(lat.measure_correlators(ld), d["corr0"], rtol)
    levels = int(d["levels"])
    if not levels:
        return
    bd = [int(k != ld) for k in range(3)]
    got = lat.measure_blocked_correlators(bd, 8, ld)
    assert len(got) == levels
    for k in range(1, levels + 1):
        corr_close(got[k - 1], d[f"b{k}_corr"], rtol)
        if precision == 64:
            sides, link, trip = lat.blocked_fields(bd, k)
            assert list(sides) == list(d[f"b{k}_L"])
            lex = lex_order(d[f"b{k}_coords"], sides)
            assert np.max(np.abs(link[lex] - d[f"b{k}_link"])) < 1e-13
            assert np.max(np.abs(trip[lex] - d[f"b{k}_trip"])) < 1e-13


def test_blocked_correlators_refused_with_doublet(gpu):
    d = load("correl_fundadj_8x6x10.npz")
    lat = lattice_of(gpu, d, 64)
    with pytest.raises(gpu.SU2GPUError):
        lat.measure_blocked_correlators([1, 1, 0], 1)


@pytest.mark.parametrize("content,L,levels", [("adj", (16, 12, 20), 2), ("fundadj", (12, 18, 10), 0),
                                             ("adj", (24, 8, 8), 2), ("fund", (10, 10, 10), 0)])
def test_correlators_match_oracle(gpu, content, L, levels):
    p = abi.make_params(content, L=L)
    f = hot_fields(p, seed=31, trip_sigma=0.6, phi_mean=0.3)
    lat = gpu.Lattice(p, seed=1)
    lat.upload(link=f.link, d0=f.d0, trip=f.trip)
    o = Oracle(p)
    o.put(f)
    ld = o.longest_dir()
    corr_close(lat.measure_correlators(ld), o.correlators(ld), 1e-12)
    if levels:
        bd = [int(k != ld) for k in range(3)]
        got = lat.measure_blocked_correlators(bd, levels, ld)
        assert len(got) == levels
        cur = o
        for k in range(levels):
            cur = cur.block(bd)
            corr_close(got[k], cur.correlators(ld), 1e-12)
