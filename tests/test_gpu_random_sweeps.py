"""Sweeps in the random_sweeps mode (update.c:278-300, 338-344 of su2higgs) on
the GPU against the oracle updating in the same order (the order stream is
shared by both): fields within 1e-9 after three sweeps, counters equal.  The
graph flag of run_sweeps is ignored in this mode (the order changes every
sweep), so run_sweeps gives the same fields as sweep-by-sweep updates."""
import numpy as np
import pytest

from native import Oracle, hot_fields
from su2higgs_gb300 import abi

pytestmark = pytest.mark.gpu

ATOL = 1e-9


@pytest.fixture(scope="module")
def gpu():
    from su2higgs_gb300 import gpu as g
    g.lib()
    return g


def upload(lat, f):
    lat.upload(link=f.link, u1=f.u1, d0=f.d0, d1=f.d1, trip=f.trip, sing=f.sing)


@pytest.mark.parametrize("content,L,over", [("su2u1s", (6, 4, 8), {}), ("adj", (8, 8, 6), {"update_links": 2}),
                                            ("fund", (8, 6, 4), {"scalar_sweeps": 3})])
def test_random_order_sweeps_match_oracle(gpu, content, L, over):
    p = abi.make_params(content, L=L, **over)
    f = hot_fields(p, seed=12, phi_mean=0.5)
    lat = gpu.Lattice(p, seed=314, chain=2)
    lat.set_random_sweeps(True)
    upload(lat, f)
    o = Oracle(p)
    o.put(f)
    o.set_random_sweeps(True)
    for s in (40, 41, 42):
        lat.update_lattice(s)
        o.set_rng(314, s, 2)
        o.update()
    got, want = lat.download(), o.get()
    for k in ("link", "u1", "d0", "d1", "trip", "sing"):
        if got[k] is not None:
            assert np.max(np.abs(got[k] - getattr(want, k))) < ATOL, k
    assert np.array_equal(lat.counters()[:22], o.counters()[:22])
    # the fixed order gives other fields
    o2 = Oracle(p)
    o2.put(f)
    for s in (40, 41, 42):
        o2.set_rng(314, s, 2)
        o2.update()
    assert np.max(np.abs(o2.get().link - want.link)) > 1e-3


def test_random_order_run_sweeps_equals_stepwise(gpu):
    p = abi.make_params("su2u1s", L=(8, 8, 8))
    f = hot_fields(p, seed=3, phi_mean=0.5)
    a = gpu.Lattice(p, seed=99)
    b = gpu.Lattice(p, seed=99)
    for lat in (a, b):
        lat.set_random_sweeps(True)
        upload(lat, f)
    a.run_sweeps(5, 4, graph=True)
    for s in range(5, 9):
        b.update_lattice(s)
    da, db = a.download(), b.download()
    for k in da:
        if da[k] is not None:
            assert np.array_equal(da[k], db[k]), k
    # switching the mode off again restores graph replay of the fixed order
    a.set_random_sweeps(False)
    b.set_random_sweeps(False)
    a.run_sweeps(9, 3, graph=True)
    for s in range(9, 12):
        b.update_lattice(s)
    assert np.array_equal(a.download()["link"], b.download()["link"])


@pytest.mark.parametrize("precision", [64, 32])
def test_clone_and_copy_fields(gpu, precision):
    """su2gpu_clone / su2gpu_copy_fields (the field copies of the heatbath
    trajectories, hb_trajectory.c:26-29, 61): a clone starts from the same
    fields, runs its own stream, and copy_fields restores it exactly."""
    p = abi.make_params("fund", L=(8, 8, 8), precision=precision)
    f = hot_fields(abi.make_params("fund", L=(8, 8, 8)), seed=4, phi_mean=0.5)
    lat = gpu.Lattice(p, seed=1)
    upload(lat, f)
    before = lat.download()
    c = lat.clone(seed=5, chain=0x40000001)
    for k, v in c.download().items():
        if v is not None:
            assert np.array_equal(v, before[k]), k
    c.set_random_sweeps(True)
    c.run_sweeps(0, 3, graph=False)
    assert not np.array_equal(c.download()["link"], before["link"])
    c.copy_fields_from(lat)
    for k, v in c.download().items():
        if v is not None:
            assert np.array_equal(v, before[k]), k
    # the source is untouched
    assert np.array_equal(lat.download()["d0"], before["d0"])
    other = gpu.Lattice(abi.make_params("fund", L=(8, 8, 6), precision=precision), seed=1)
    with pytest.raises(gpu.SU2GPUError):
        other.copy_fields_from(lat)
    c.close()
    other.close()
