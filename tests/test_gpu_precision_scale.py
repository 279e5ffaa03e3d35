"""Precision at scale: the FP32 form against the FP64 path and the oracle on
large lattices, from one checkpoint.

SU(2) + fundamental Higgs at beta 8, m^2 -0.1, lambda 0.002.  A seeded hot
start is brought to equilibrium by the FP64 GPU path; from that checkpoint
four FP32 and four FP64 chains run on the GPU (independent random streams)
and, at 64^3, oracle chains (FP64, CPU) run in worker processes.  Plaquette,
phi^2 and the hopping term must agree within 3 sigma of binned jackknife
errors; each difference is printed with its error.  At 128^3 the GPU FP32
chain is compared with the GPU FP64 chain only (an oracle sweep of 128^3
takes seconds).  The FP32 form re-normalises every link it writes, which
subsumes a periodic re-unitarisation.
"""
import numpy as np
import pytest

from native import hot_fields
from su2higgs_gb300 import abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from su2higgs_gb300 import gpu as g
    g.lib()
    return g


def gpu_series(gpu, p, start, seed, n):
    import chains
    names = chains.CONTENT_OBSERVABLES["fund"]
    lat = gpu.Lattice(p, seed=seed)
    lat.upload(**start)
    V = p.sites()
    rows = []
    for s in range(n):
        lat.run_sweeps(s, 1, graph=True)
        rows.append(chains.observables(names, lat.measure(), V, p.betasu2))
    lat.close()
    return np.array(rows)


def checkpoint(gpu, L, ntherm):
    p64 = abi.make_params("fund", L=L)
    f = hot_fields(p64, seed=64, phi_mean=1.0)
    lat = gpu.Lattice(p64, seed=6464)
    lat.upload(link=f.link, d0=f.d0)
    lat.run_sweeps(0, ntherm, graph=True)
    out = lat.download()
    lat.close()
    return {"link": out["link"], "d0": out["d0"]}


@pytest.mark.parametrize("side", [64, 128])
def test_fp32_against_fp64_and_oracle_at_scale(gpu, side):
    import chains
    L = (side,) * 3
    start = checkpoint(gpu, L, 400)
    n = 2000 if side == 64 else 800
    sets = {"fp32": [gpu_series(gpu, abi.make_params("fund", L=L, precision=32), start, 32 + k, n)
                     for k in range(4)],
            "fp64": [gpu_series(gpu, abi.make_params("fund", L=L, precision=64), start, 64 + k, n)
                     for k in range(4)]}
    if side == 64:
        # oracle chains of 60 sweeps from the checkpoint, the first 10 left
        # out (they still remember the common start)
        orc = chains.oracle_chains("fund", L, {}, [start] * 12, 777, 10, 50)
        sets["oracle"] = orc
    names = chains.CONTENT_OBSERVABLES["fund"]
    rows, fails = chains.compare(names, sets)
    print("\n" + chains.format_rows(f"fundamental {side}^3 from one checkpoint", rows))
    assert not fails, fails
