"""Profiles along the z direction (measure_along_z, z_coord.c:206-300) on the
GPU against the oracle: the z direction (the longest one, ties to the last,
init_z_coord z_coord.c:18-24) and the plane sums of phi^2, Tr Sigma^2, S and
S^2, 1e-12 relative in FP64 (the summation order differs), 1e-5 in the FP32
form."""
import numpy as np
import pytest

from native import Oracle, hot_fields
from su2higgs_gb300 import abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from su2higgs_gb300 import gpu as g
    g.lib()
    return g


@pytest.mark.parametrize("precision,rtol", [(64, 1e-12), (32, 1e-5)])
@pytest.mark.parametrize("content,L,zdir", [("su2u1s", (6, 4, 8), 2), ("fundadj", (10, 4, 6), 0),
                                           ("su2u1s", (4, 12, 6), 1), ("adj", (8, 8, 8), 2),
                                           ("fund", (8, 6, 8), 2)])
def test_measure_z_matches_oracle(gpu, content, L, zdir, precision, rtol):
    p = abi.make_params(content, L=L, precision=precision)
    p64 = abi.make_params(content, L=L)
    f = hot_fields(p64, seed=9, phi_mean=0.5)
    lat = gpu.Lattice(p, seed=1)
    lat.upload(link=f.link, u1=f.u1, d0=f.d0, trip=f.trip, sing=f.sing)
    zd, got = lat.measure_z()
    o = Oracle(p64)
    o.put(f)
    ozd, want = o.measure_z()
    assert zd == ozd == zdir
    assert got.shape == (L[zdir], 4)
    assert np.allclose(got, want, rtol=rtol, atol=1e-300)
    # the plane sums add up to the volume sums of measure()
    m = lat.measure()
    if p.nhiggs() > 0:
        assert abs(got[:, 0].sum() - m[abi.M_PHI2]) < 1e-9 * abs(m[abi.M_PHI2]) + 1e-12
    if p.content & abi.TRIPLET:
        assert abs(got[:, 1].sum() - m[abi.M_SIGMA2]) < 1e-9 * abs(m[abi.M_SIGMA2]) + 1e-12
