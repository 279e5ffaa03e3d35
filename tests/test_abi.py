"""CPU checks of the C ABI: the library exports every entry point that
include/su2gpu.h declares, and its host-side random stream is the Philox
stream of the oracle, which in turn reproduces the published Random123
known-answer vectors of Philox4x32-10.  No compute call needs a GPU here."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from native import ROOT, oracle_lib
from su2higgs_gb300 import abi

HEADER = os.path.join(ROOT, "include", "su2gpu.h")


def declared_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(su2gpu_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def libpath():
    from su2higgs_gb300 import build
    return build.build()


def test_library_exports_every_declared_symbol(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (su2gpu_[a-z0-9_]+)", out))
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing
    assert len(declared_functions()) >= 20


def test_library_loads_and_reports_version(libpath):
    from su2higgs_gb300 import gpu
    assert gpu.lib().su2gpu_version() >= 10000


def test_struct_layout_matches_header(libpath):
    # su2gpu_params: 20 int32 then 26 doubles; su2gpu_weight: 8 int32, 7 doubles, 8 pointers
    assert ctypes.sizeof(abi.Params) == 20 * 4 + 26 * 8
    assert ctypes.sizeof(abi.Weight) == 8 * 4 + 7 * 8 + 8 * ctypes.sizeof(ctypes.c_void_p)


@pytest.mark.parametrize("ctr,key,expect", [
    ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
    ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
     [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
])
def test_philox_known_answers(ctr, key, expect):
    L = oracle_lib()
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    L.orc_philox_raw(c, k, o)
    assert list(o) == expect


def test_product_stream_equals_oracle_stream(libpath):
    from su2higgs_gb300 import gpu
    L = oracle_lib()
    L.orc_stream_uniform_at.restype = ctypes.c_double
    L.orc_stream_uniform_at.argtypes = [ctypes.c_uint64] + [ctypes.c_uint32] * 5
    rng = np.random.default_rng(7)
    for _ in range(3000):
        seed = int(rng.integers(0, 2 ** 63))
        site = int(rng.integers(0, 2 ** 32))
        ps = int(rng.integers(0, 65536))
        d = int(rng.integers(0, 64))
        sw = int(rng.integers(0, 2 ** 32))
        ch = int(rng.integers(0, 2 ** 32))
        a = L.orc_stream_uniform_at(seed, site, ps, d, sw, ch)
        b = gpu.stream_uniform(seed, site, ps, d, sw, ch)
        assert a == b
        assert 0.0 <= b < 1.0


def test_invalid_params_rejected_without_gpu(libpath):
    from su2higgs_gb300 import gpu
    p = abi.make_params("fund", L=(7, 8, 8))
    assert gpu.lib().su2gpu_footprint_bytes(ctypes.byref(p)) == -1
    p = abi.make_params("fund", L=(8, 8, 8))
    assert gpu.lib().su2gpu_footprint_bytes(ctypes.byref(p)) > 8 * 8 * 8 * 3 * 32
