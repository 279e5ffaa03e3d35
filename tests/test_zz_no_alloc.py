"""su2gpu_measure_noalloc: the measurement entry point for callers that
cannot allocate device memory (an embedding framework whose allocator owns
the device memory, or a loop that must not risk the synchronisation of a
cudaMalloc).  It takes the caller's device buffers for the fields and the
result and uses only a file-scope scratch array.

The test gives it fields laid out as the library keeps them, calls it twice in
a row (the second call reuses the shared scratch), and checks both results
against su2gpu_measure on the same fields, with the 1e-12 relative tolerance
of the other measurement tests, and on configurations of the reference's own
runs against the reference's measure() sums.  It also checks that a lattice
beyond the scratch limit (128^3 sites) is refused.  This file is collected
last.
"""
import ctypes

import numpy as np
import pytest

from golden_io import measure_close
from native import hot_fields
from su2higgs_gb300 import abi

pytestmark = pytest.mark.gpu

RTOL = 1e-12
# FP32 fields: the allocation-free kernel is the content-generic instantiation
# of the per-site measurement, `measure` the content-specialised one; the
# compiler may fuse their multiply-adds differently, so a site's FP32 value
# can differ in its last bit (one site in ~2000 moves a sum by ~5e-11)
RTOL32 = 2e-6


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    from su2higgs_gb300 import gpu
    L = gpu.lib()
    L.su2gpu_measure_noalloc.argtypes = [ctypes.POINTER(abi.Params), ctypes.POINTER(abi.DeviceFields),
                                         ctypes.c_void_p, ctypes.c_void_p]
    return torch, gpu, L


def device_layout(torch, f, precision):
    """The fields as the library keeps them on the device: parity-split
    structure of arrays (host arrays are already in the EVEN-first order)."""
    dt = torch.float64 if precision == 64 else torch.float32
    dev = torch.device("cuda")
    keep = []

    def put(a):
        t = torch.tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
        keep.append(t)
        return t.data_ptr()

    df = abi.DeviceFields()
    for d in range(3):
        df.link[d] = put(f.link[:, d, :])
        if f.u1 is not None:
            df.u1[d] = put(f.u1[:, d])
        if f.trip is not None:
            df.triplet[d] = put(f.trip[:, d])
    if f.d0 is not None:
        df.doublet[0] = put(f.d0)
    if f.d1 is not None:
        df.doublet[1] = put(f.d1)
    if f.sing is not None:
        df.singlet = put(f.sing)
    return df, keep


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("content", ["fund", "adj", "su2u1s", "higgs2"])
def test_noalloc_measure_matches_measure(env, content, precision):
    torch, gpu, L = env
    p = abi.make_params(content, L=(16, 12, 10), precision=precision)
    f = hot_fields(p, seed=31, phi_mean=0.5)
    lat = gpu.Lattice(p)
    lat.upload(link=f.link, u1=f.u1, d0=f.d0, d1=f.d1, trip=f.trip, sing=f.sing)
    want = lat.measure()
    df, keep = device_layout(torch, f, precision)
    out = torch.full((2, abi.NMEAS), float("nan"), dtype=torch.float64, device="cuda")
    for k in range(2):
        rc = L.su2gpu_measure_noalloc(ctypes.byref(p), ctypes.byref(df), ctypes.c_void_p(out[k].data_ptr()), None)
        assert rc == abi.OK, L.su2gpu_last_error().decode()
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    for k in range(2):
        ok, idx, a, b = measure_close(got[k], want, RTOL if precision == 64 else RTOL32)
        assert ok, (k, idx, a, b)
    assert np.array_equal(got[0], got[1])
    del keep


def test_noalloc_rejects_lattices_beyond_its_scratch(env):
    torch, gpu, L = env
    p = abi.make_params("fund", L=(130, 128, 128))
    df = abi.DeviceFields()
    out = torch.zeros(abi.NMEAS, dtype=torch.float64, device="cuda")
    rc = L.su2gpu_measure_noalloc(ctypes.byref(p), ctypes.byref(df), ctypes.c_void_p(out.data_ptr()), None)
    assert rc == abi.ERR_CAPACITY
    assert "2097152" in L.su2gpu_last_error().decode()


@pytest.mark.parametrize("name", ["sites_fund.npz", "sites_adj.npz", "sites_su2u1s.npz", "sites_higgs2.npz",
                                  "sites_fundadj.npz"])
def test_noalloc_measure_matches_reference_sums(env, name):
    """On a configuration of the reference's own run, two calls in a row give
    the reference's measure() sums (measure.c:110-233) within 1e-12."""
    from golden_io import fields_of, load, params_of
    torch, gpu, L = env
    d = load(name)
    p = params_of(d)
    f = fields_of(d, p, "in_")
    df, keep = device_layout(torch, f, 64)
    out = torch.full((2, abi.NMEAS), float("nan"), dtype=torch.float64, device="cuda")
    for k in range(2):
        rc = L.su2gpu_measure_noalloc(ctypes.byref(p), ctypes.byref(df), ctypes.c_void_p(out[k].data_ptr()), None)
        assert rc == abi.OK, L.su2gpu_last_error().decode()
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    for k in range(2):
        ok, idx, a, b = measure_close(got[k], d["measure"], RTOL)
        assert ok, (k, idx, a, b)
    del keep
