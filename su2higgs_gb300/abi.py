"""ctypes mirror of the C ABI in include/su2gpu.h.

The structures here are the exact in-memory layout of ``su2gpu_params`` and
``su2gpu_weight``; the constants mirror the reference's compile-time flags
(su2higgs Makefile:3-16), update algorithms (generic/stddefs.h:47-49) and
multicanonical settings (stddefs.h:57-65).
"""
import ctypes

# field content bits
HIGGS1 = 0x01
HIGGS2 = 0x02
TRIPLET = 0x04
SINGLET = 0x08
U1 = 0x10
GRADFLOW = 0x20

# named contents used across the project (the reference's -D sets)
CONTENTS = {
    "pure": 0,
    "fund": HIGGS1,
    "adj": TRIPLET,
    "su2u1s": HIGGS1 | SINGLET | U1,
    "fundadj": HIGGS1 | TRIPLET,
    "higgs2": HIGGS2 | U1,
}

METROPOLIS = 1
HEATBATH = 2
OVERRELAX = 3

PHISQ = 1
SIGMASQ = 2
PHI2MINUSSIGMA2 = 3
PHI2SQ = 4
MUCA_READONLY = 0
MUCA_FAST = 1
MUCA_SLOW = 2

OK = 0
ERR_INVALID = -1
ERR_CUDA = -2
ERR_NOMEM = -3
ERR_UNSUPPORTED = -4
ERR_KERNEL = -5
ERR_CAPACITY = -6

# counters (su2.h:208-231)
C_TOTAL_SU2LINK, C_ACC_SU2LINK = 0, 1
C_TOTAL_U1LINK, C_ACC_U1LINK = 2, 3
C_TOTAL_DOUBLET, C_ACC_DOUBLET = 4, 6
C_TOTAL_OR_DOUBLET, C_ACC_OR_DOUBLET = 8, 10
C_TOTAL_TRIPLET, C_ACC_TRIPLET = 12, 13
C_TOTAL_OR_TRIPLET, C_ACC_OR_TRIPLET = 14, 15
C_TOTAL_SINGLET, C_ACC_SINGLET = 16, 17
C_TOTAL_OR_SINGLET, C_ACC_OR_SINGLET = 18, 19
C_TOTAL_MUCA, C_ACC_MUCA = 20, 21
C_KP_CAP, C_POLY_FALLBACK = 22, 23
NCOUNTERS = 24

# measure() volume sums
M_ACTION, M_WILSON, M_U1WILSON = 0, 1, 2
M_COV_PHI, M_PHI2, M_PHI4 = 3, 4, 5  # + 3*higgs_id
M_PHI12_RE, M_PHI12_IM = 9, 10
M_HOP_SIGMA, M_SIGMA2, M_SIGMA4, M_PHI2SIGMA2 = 11, 12, 13, 14
M_MAGCHARGE, M_MAGCHARGE_ABS = 15, 16
M_S_COV, M_S1, M_S2, M_S3, M_S4, M_SPHI2, M_S2PHI2 = 17, 18, 19, 20, 21, 22, 23
NMEAS = 24
# correlator columns (SU2GPU_CORR_*): Higgs, Sigma^2, photon (1,0), (2,0),
# (1,1), (2,1) re/im
NCORR = 10


class Params(ctypes.Structure):
    """su2gpu_params: couplings and update recipe (reference params, su2.h:76-181)."""

    _fields_ = [
        ("dim", ctypes.c_int32),
        ("L", ctypes.c_int32 * 4),
        ("content", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("algorithm_su2link", ctypes.c_int32),
        ("algorithm_u1link", ctypes.c_int32),
        ("algorithm_su2doublet", ctypes.c_int32),
        ("algorithm_su2triplet", ctypes.c_int32),
        ("algorithm_singlet", ctypes.c_int32),
        ("update_links", ctypes.c_int32),
        ("scalar_sweeps", ctypes.c_int32),
        ("update_su2doublet", ctypes.c_int32),
        ("update_su2triplet", ctypes.c_int32),
        ("update_singlet", ctypes.c_int32),
        ("reunitarize_interval", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 2),
        ("betasu2", ctypes.c_double),
        ("msq_phi", ctypes.c_double),
        ("lambda_phi", ctypes.c_double),
        ("msq_triplet", ctypes.c_double),
        ("a2", ctypes.c_double),
        ("b4", ctypes.c_double),
        ("betau1", ctypes.c_double),
        ("r_u1", ctypes.c_double),
        ("b1_s", ctypes.c_double),
        ("msq_s", ctypes.c_double),
        ("b3_s", ctypes.c_double),
        ("b4_s", ctypes.c_double),
        ("a1_s", ctypes.c_double),
        ("a2_s", ctypes.c_double),
        ("msq_phi2", ctypes.c_double),
        ("m12sq_re", ctypes.c_double),
        ("m12sq_im", ctypes.c_double),
        ("lam2", ctypes.c_double),
        ("lam3", ctypes.c_double),
        ("lam4", ctypes.c_double),
        ("lam5_re", ctypes.c_double),
        ("lam5_im", ctypes.c_double),
        ("lam6_re", ctypes.c_double),
        ("lam6_im", ctypes.c_double),
        ("lam7_re", ctypes.c_double),
        ("lam7_im", ctypes.c_double),
    ]

    def sites(self):
        v = 1
        for d in range(self.dim):
            v *= self.L[d]
        return v

    def nhiggs(self):
        return 2 if self.content & HIGGS2 else (1 if self.content & HIGGS1 else 0)


class Weight(ctypes.Structure):
    """su2gpu_weight: multicanonical weight (reference weight, su2.h:235-274)."""

    _fields_ = [
        ("orderparam", ctypes.c_int32),
        ("mode", ctypes.c_int32),
        ("do_acceptance", ctypes.c_int32),
        ("checks_per_sweep", ctypes.c_int32),
        ("bins", ctypes.c_int32),
        ("muca_count", ctypes.c_int32),
        ("update_interval", ctypes.c_int32),
        ("last_max", ctypes.c_int32),
        ("param_value", ctypes.c_double * 2),
        ("min", ctypes.c_double),
        ("max", ctypes.c_double),
        ("wrk_min", ctypes.c_double),
        ("wrk_max", ctypes.c_double),
        ("delta", ctypes.c_double),
        ("pos", ctypes.POINTER(ctypes.c_double)),
        ("W", ctypes.POINTER(ctypes.c_double)),
        ("slope", ctypes.POINTER(ctypes.c_double)),
        ("b", ctypes.POINTER(ctypes.c_double)),
        ("hits", ctypes.POINTER(ctypes.c_int32)),
        ("gsum", ctypes.POINTER(ctypes.c_int64)),
        ("nsum", ctypes.POINTER(ctypes.c_int64)),
        ("hgram", ctypes.POINTER(ctypes.c_double)),
    ]


class DeviceFields(ctypes.Structure):
    """su2gpu_device_fields: device pointers in the library's field layout."""

    _fields_ = [
        ("link", ctypes.c_void_p * 3),
        ("u1", ctypes.c_void_p * 3),
        ("doublet", ctypes.c_void_p * 2),
        ("triplet", ctypes.c_void_p * 3),
        ("singlet", ctypes.c_void_p),
    ]


def make_params(content="fund", L=(8, 8, 8), precision=64, **kw):
    """Parameters with the reference config's defaults (su2higgs config:1-156)
    overridden by keyword arguments; `content` is a name or a bit mask."""
    p = Params()
    p.dim = len(L)
    for d, n in enumerate(L):
        p.L[d] = n
    p.content = CONTENTS[content] if isinstance(content, str) else int(content)
    p.precision = precision
    p.algorithm_su2link = HEATBATH
    p.algorithm_u1link = METROPOLIS
    p.algorithm_su2doublet = OVERRELAX
    p.algorithm_su2triplet = OVERRELAX
    p.algorithm_singlet = OVERRELAX
    p.update_links = 1
    p.scalar_sweeps = 4
    p.update_su2doublet = 1
    p.update_su2triplet = 1
    p.update_singlet = 1
    p.reunitarize_interval = 10
    p.betasu2 = 8.0
    p.msq_phi = -0.10
    p.lambda_phi = 0.002
    p.msq_triplet = -0.5032354703283564
    p.a2 = 2.6953060227675745
    p.b4 = 0.11666666666666665
    p.betau1 = 24.0
    p.r_u1 = 1.0
    p.b1_s = 0.0
    p.msq_s = -0.1
    p.b3_s = 0.0
    p.b4_s = 0.3
    p.a1_s = 0.0
    p.a2_s = 0.25
    p.msq_phi2 = 0.2
    p.m12sq_re, p.m12sq_im = 0.04, 0.06
    p.lam2, p.lam3, p.lam4 = 0.02, 0.03, 0.04
    p.lam5_re, p.lam5_im = 0.05, 0.055
    p.lam6_re, p.lam6_im = 0.006, 0.0065
    p.lam7_re, p.lam7_im = 0.007, 0.0075
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p
