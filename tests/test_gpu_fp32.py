"""The FP32 precision form: FP32 fields, FP64 volume sums and multicanonical
decisions.  Checked against the reference's FP64 outputs and the FP64 GPU path
with FP32-sized tolerances (stated per test)."""
import numpy as np
import pytest

from golden_io import fields_of, load, names, params_of
from native import hot_fields
from su2higgs_gb300 import abi

pytestmark = pytest.mark.gpu

# per-site arithmetic in FP32 (rounding 6e-8), summed in FP64
RTOL_MEAS = 2e-5


@pytest.fixture(scope="module")
def gpu():
    from su2higgs_gb300 import gpu as g
    g.lib()
    return g


def upload(lat, f):
    lat.upload(link=f.link, u1=f.u1, d0=f.d0, d1=f.d1, trip=f.trip, sing=f.sing)


@pytest.mark.parametrize("name", names("sites_"))
def test_fp32_measure_close_to_reference(gpu, name):
    d = load(name)
    p = params_of(d)
    p.precision = 32
    lat = gpu.Lattice(p)
    upload(lat, fields_of(d, p, "in_"))
    m = lat.measure()
    ref = d["measure"]
    for k in range(abi.NMEAS):
        if k == abi.M_MAGCHARGE:
            assert abs(m[k] - ref[k]) < 1e-3 * max(1.0, ref[abi.M_MAGCHARGE_ABS]), k
        elif ref[k] != 0:
            scale = max(abs(ref[k]), 1e-3 * abs(ref[abi.M_ACTION]))
            assert abs(m[k] - ref[k]) <= RTOL_MEAS * scale, (k, m[k], ref[k])


def test_fp32_links_stay_unitary(gpu):
    p = abi.make_params("fund", L=(16, 16, 16), precision=32, algorithm_su2link=abi.METROPOLIS)
    f = hot_fields(p, seed=2)
    lat = gpu.Lattice(p, seed=4)
    upload(lat, f)
    lat.run_sweeps(0, 30, graph=True)
    n = np.linalg.norm(lat.download()["link"], axis=2)
    assert np.max(np.abs(n - 1.0)) < 1e-6


def test_fp32_graph_equals_stepwise(gpu):
    p = abi.make_params("su2u1s", L=(8, 8, 8), precision=32)
    f = hot_fields(p, seed=6, phi_mean=0.5)
    a, b = gpu.Lattice(p, seed=1), gpu.Lattice(p, seed=1)
    upload(a, f)
    upload(b, f)
    for s in range(4):
        a.update_lattice(s)
    b.run_sweeps(0, 4, graph=True)
    fa, fb = a.download(), b.download()
    for n in fa:
        if fa[n] is not None:
            assert np.array_equal(fa[n], fb[n]), n
