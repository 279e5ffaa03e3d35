"""measure_local (measure.c:368-487) on the GPU against the oracle: per site,
in storage order, Tr Sigma^2 and the magnetic charge magcharge_cube /
(2 pi sqrt(beta)) (magfield.c:262-280).  FP64: 1e-12 relative for Tr Sigma^2,
1e-10 absolute for the charge (a sum of atan2 angles, an integer in exact
arithmetic); FP32 form: 1e-5 relative and 1e-3 absolute.  The charges are
integers, and their magnitudes sum to the measure() monopole count."""
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


@pytest.mark.parametrize("precision,rtol,atol", [(64, 1e-12, 1e-10), (32, 1e-5, 1e-3)])
@pytest.mark.parametrize("content,L", [("adj", (8, 6, 10)), ("fundadj", (6, 6, 6))])
def test_measure_local_matches_oracle(gpu, content, L, precision, rtol, atol):
    p = abi.make_params(content, L=L, precision=precision, betasu2=5.0)
    p64 = abi.make_params(content, L=L, betasu2=5.0)
    f = hot_fields(p64, seed=44, phi_mean=0.3)
    lat = gpu.Lattice(p, seed=1)
    lat.upload(link=f.link, d0=f.d0, trip=f.trip)
    got = lat.measure_local()
    o = Oracle(p64)
    o.put(f)
    want = o.measure_local()
    assert np.allclose(got[:, 0], want[:, 0], rtol=rtol, atol=0)
    assert np.max(np.abs(got[:, 1] - want[:, 1])) < atol
    assert np.max(np.abs(want[:, 1] - np.round(want[:, 1]))) < 1e-9
    assert np.any(np.round(want[:, 1]) != 0)  # a hot lattice has monopoles
    m = lat.measure()
    assert abs(m[abi.M_MAGCHARGE_ABS] / (2 * np.pi * np.sqrt(5.0)) - np.sum(np.abs(got[:, 1]))) < 1e-6 * len(got)


def test_flow_local_first_equals_measure_local(gpu):
    p = abi.make_params("adj", L=(8, 8, 8), betasu2=6.0)
    f = hot_fields(p, seed=45, phi_mean=0.3)
    lat = gpu.Lattice(p, seed=1)
    lat.upload(link=f.link, trip=f.trip)
    rows, local = lat.grad_flow_local(0.2, 0.05, 2)
    assert local.shape == (rows.shape[0], p.sites(), 2)
    assert np.array_equal(local[0], lat.measure_local())  # t = 0 is the unflowed lattice
    plain = lat.grad_flow(0.2, 0.05, 2)
    assert np.array_equal(rows, plain)
