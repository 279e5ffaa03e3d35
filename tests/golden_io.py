"""Loading helpers for the golden fixtures (tests/golden/*.npz)."""
import glob
import os

import numpy as np

from native import Fields, WeightBuf
from su2higgs_gb300 import abi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


def names(prefix):
    return sorted(os.path.basename(x) for x in glob.glob(os.path.join(GOLDEN, prefix + "*.npz")))


def params_of(d):
    p = abi.Params()
    for name, _ in abi.Params._fields_:
        if name == "reserved":
            continue
        v = d["p_" + name]
        if name == "L":
            for k, x in enumerate(v):
                p.L[k] = int(x)
        elif isinstance(getattr(p, name), int):
            setattr(p, name, int(v))
        else:
            setattr(p, name, float(v))
    return p


def fields_of(d, p, prefix):
    kw = {}
    for name in ("link", "u1", "d0", "d1", "trip", "sing"):
        if prefix + name in d:
            kw[name] = d[prefix + name]
    return Fields(p, **kw)


def weight_of(d, prefix):
    bins = int(d[prefix + "bins"])
    w = WeightBuf(bins, orderparam=int(d[prefix + "orderparam"]), mode=int(d[prefix + "mode"]),
                  checks_per_sweep=int(d[prefix + "checks_per_sweep"]))
    for k in ("pos", "W", "slope", "b", "hits"):
        getattr(w, k)[:] = d[prefix + k]
    for k in ("gsum", "nsum", "hgram"):  # the SLOW mode's accumulators
        if prefix + k in d:
            getattr(w, k)[:] = d[prefix + k]
    s = w.struct
    for k in ("min", "max", "wrk_min", "wrk_max", "delta"):
        setattr(s, k, float(d[prefix + k]))
    s.last_max = int(d[prefix + "last_max"])
    s.muca_count = int(d[prefix + "muca_count"])
    s.update_interval = int(d[prefix + "update_interval"])
    pv = d[prefix + "param_value"]
    s.param_value[0], s.param_value[1] = float(pv[0]), float(pv[1])
    return w


def measure_close(a, b, rtol=1e-12):
    """Compare two SU2GPU_M_* vectors.  The total magnetic charge is a
    telescoping sum that is zero in exact arithmetic, so it is compared with an
    absolute tolerance scaled by the charge-magnitude sum."""
    a = np.asarray(a)
    b = np.asarray(b)
    for k in range(abi.NMEAS):
        if k == abi.M_MAGCHARGE:
            tol = rtol * max(abs(b[abi.M_MAGCHARGE_ABS]), 1.0) * 100
        else:
            tol = rtol * max(abs(a[k]), abs(b[k]), 1e-300)
        if abs(a[k] - b[k]) > tol:
            return False, k, a[k], b[k]
    return True, None, None, None
