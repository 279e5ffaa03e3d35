"""Test-side access to the oracle (oracle/liboracle.so) and, when it was built
in this checkout, the reference harness (oracle/_ref/libref_<content>.so).

Both take FP64 AoS field arrays in the reference's layout site order.
"""
import ctypes
import os
import subprocess
import tempfile

import numpy as np

from su2higgs_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
REF_DIR = os.path.join(ORACLE_DIR, "_ref")

_P = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731


def build_oracle():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


_oracle = None


def oracle_lib():
    global _oracle
    if _oracle is None:
        path = os.path.join(ORACLE_DIR, "liboracle.so")
        if not os.path.exists(path):
            build_oracle()
        lib = ctypes.CDLL(path)
        lib.orc_create.restype = ctypes.c_void_p
        lib.orc_create.argtypes = [ctypes.POINTER(abi.Params)]
        for name in ("orc_destroy", "orc_update_lattice", "orc_reset_counters", "orc_muca_init_last_max"):
            getattr(lib, name).argtypes = [ctypes.c_void_p]
        lib.orc_sites.restype = ctypes.c_long
        lib.orc_sites.argtypes = [ctypes.c_void_p]
        lib.orc_set_rng.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32]
        lib.orc_site_update.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_long, ctypes.c_int, ctypes.c_uint32]
        lib.orc_site_draws.argtypes = [ctypes.c_void_p]
        lib.orc_or_proposal.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_long, ctypes.c_int, ctypes.c_void_p]
        for name in ("orc_localact_su2link", "orc_localact_u1link"):
            getattr(lib, name).restype = ctypes.c_double
            getattr(lib, name).argtypes = [ctypes.c_void_p, ctypes.c_long, ctypes.c_int]
        for name in ("orc_local_su2wilson", "orc_action_local", "orc_local_u1wilson", "orc_localact_triplet",
                     "orc_localact_singlet", "orc_magcharge_cube"):
            getattr(lib, name).restype = ctypes.c_double
            getattr(lib, name).argtypes = [ctypes.c_void_p, ctypes.c_long]
        lib.orc_localact_doublet.restype = ctypes.c_double
        lib.orc_localact_doublet.argtypes = [ctypes.c_void_p, ctypes.c_long, ctypes.c_int]
        lib.orc_alpha_proj.restype = ctypes.c_double
        lib.orc_alpha_proj.argtypes = [ctypes.c_void_p, ctypes.c_long, ctypes.c_int, ctypes.c_int]
        for name in ("orc_wilson_staple", "orc_link_staple", "orc_staple_doublet"):
            getattr(lib, name).argtypes = [ctypes.c_void_p, ctypes.c_long, ctypes.c_int, ctypes.c_void_p]
        lib.orc_polysolve3.restype = ctypes.c_double
        lib.orc_polysolve3.argtypes = [ctypes.c_double] * 4
        lib.orc_calc_orderparam.restype = ctypes.c_double
        lib.orc_calc_orderparam.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.orc_get_weight.restype = ctypes.c_double
        lib.orc_get_weight.argtypes = [ctypes.c_void_p, ctypes.c_double]
        lib.orc_whichbin.argtypes = [ctypes.c_void_p, ctypes.c_double]
        lib.orc_muca_set.argtypes = [ctypes.c_void_p, ctypes.POINTER(abi.Weight)]
        lib.orc_muca_get.argtypes = [ctypes.c_void_p, ctypes.POINTER(abi.Weight)]
        lib.orc_flow_step.argtypes = [ctypes.c_void_p, ctypes.c_double]
        lib.orc_grad_flow.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                      ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        # the handle is a 64-bit pointer: never let ctypes pass it as a C int
        for name in ("orc_put_fields", "orc_get_fields"):
            getattr(lib, name).argtypes = [ctypes.c_void_p] * 7
        for name in ("orc_counters", "orc_measure", "orc_measure_local"):
            getattr(lib, name).argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        lib.orc_measure_z.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_void_p]
        lib.orc_set_random_sweeps.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.orc_correlators.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        lib.orc_block.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        lib.orc_sweep_order.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        _oracle = lib
    return _oracle


class Fields:
    """FP64 AoS host fields in layout order (the lattice-file field blocks)."""

    def __init__(self, p, link=None, u1=None, d0=None, d1=None, trip=None, sing=None):
        V, D = p.sites(), p.dim
        self.V, self.D = V, D
        self.link = np.zeros((V, D, 4)) if link is None else np.ascontiguousarray(link, dtype=np.float64)
        if link is None:
            self.link[..., 0] = 1.0
        nh = p.nhiggs()
        self.u1 = (np.zeros((V, D)) if u1 is None else np.ascontiguousarray(u1)) if p.content & abi.U1 else None
        self.d0 = (np.zeros((V, 4)) if d0 is None else np.ascontiguousarray(d0)) if nh > 0 else None
        self.d1 = (np.zeros((V, 4)) if d1 is None else np.ascontiguousarray(d1)) if nh > 1 else None
        self.trip = (np.zeros((V, 3)) if trip is None else np.ascontiguousarray(trip)) if p.content & abi.TRIPLET else None
        self.sing = (np.zeros((V,)) if sing is None else np.ascontiguousarray(sing)) if p.content & abi.SINGLET else None

    def arrays(self):
        return [self.link, self.u1, self.d0, self.d1, self.trip, self.sing]

    def ptrs(self):
        return [_P(a) for a in self.arrays()]

    def copy(self):
        f = Fields.__new__(Fields)
        f.V, f.D = self.V, self.D
        for name in ("link", "u1", "d0", "d1", "trip", "sing"):
            a = getattr(self, name)
            setattr(f, name, None if a is None else a.copy())
        return f

    def max_abs_diff(self, other):
        out = {}
        for name in ("link", "u1", "d0", "d1", "trip", "sing"):
            a, b = getattr(self, name), getattr(other, name)
            if a is not None:
                out[name] = float(np.max(np.abs(a - b)))
        return out


def hot_fields(p, seed=1, phi_sigma=0.1, trip_sigma=0.3, sing_sigma=0.3, u1_sigma=0.5, phi_mean=0.0):
    """Seeded hot start: Haar-random links (4 normals normalised), scalars normal."""
    rng = np.random.default_rng(seed)
    V, D = p.sites(), p.dim
    link = rng.normal(size=(V, D, 4))
    link /= np.linalg.norm(link, axis=2, keepdims=True)
    f = Fields(p, link=link)
    if f.u1 is not None:
        f.u1 = rng.normal(scale=u1_sigma, size=(V, D))
    if f.d0 is not None:
        f.d0 = rng.normal(scale=phi_sigma, size=(V, 4))
        f.d0[:, 0] += phi_mean
    if f.d1 is not None:
        f.d1 = rng.normal(scale=phi_sigma, size=(V, 4))
    if f.trip is not None:
        f.trip = rng.normal(scale=trip_sigma, size=(V, 3))
    if f.sing is not None:
        f.sing = rng.normal(scale=sing_sigma, size=(V,))
    return f


class Oracle:
    """One lattice in the C restatement (oracle/src/oracle.c)."""

    def __init__(self, p):
        self.lib = oracle_lib()
        self.p = p
        self.h = self.lib.orc_create(ctypes.byref(p))
        self.V = self.lib.orc_sites(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    def tables(self):
        V, D = self.V, self.p.dim
        nx, pv, co = (np.zeros(V * D, np.int64) for _ in range(3))
        par = np.zeros(V, np.int32)
        self.lib.orc_tables(self.h, _P(nx), _P(pv), _P(co), _P(par))
        return nx.reshape(V, D), pv.reshape(V, D), co.reshape(V, D), par

    def put(self, f):
        self.lib.orc_put_fields(self.h, *f.ptrs())

    def get(self):
        f = Fields(self.p)
        self.lib.orc_get_fields(self.h, *f.ptrs())
        return f

    def set_rng(self, seed, sweep, chain=0):
        self.lib.orc_set_rng(self.h, seed, sweep, chain)

    def set_random_sweeps(self, on=True):
        self.lib.orc_set_random_sweeps(self.h, 1 if on else 0)

    def longest_dir(self):
        """make_misc_tables (layout.c:773-777): the longest direction, ties to
        the last."""
        ld = self.p.dim - 1
        for d in range(self.p.dim - 1, -1, -1):
            if self.p.L[d] > self.p.L[ld]:
                ld = d
        return ld

    def correlators(self, dir):
        out = np.zeros((self.p.L[dir] // 2 + 1, 10))
        n = self.lib.orc_correlators(self.h, dir, _P(out))
        return out[:n].copy()

    def block(self, block_dir):
        """A new oracle lattice: this one smeared and blocked in the
        directions block_dir[d] != 0."""
        bd = np.ascontiguousarray(block_dir, dtype=np.int32)
        L = tuple(self.p.L[d] // 2 if bd[d] else self.p.L[d] for d in range(self.p.dim))
        q = abi.make_params(self.p.content, L=L)
        for name, _ in abi.Params._fields_:
            if name not in ("L", "dim"):
                setattr(q, name, getattr(self.p, name))
        out = Oracle(q)
        assert self.lib.orc_block(self.h, _P(bd), out.h) == 0
        return out

    def update(self):
        return self.lib.orc_update_lattice(self.h)

    def counters(self):
        c = np.zeros(abi.NCOUNTERS, np.int64)
        self.lib.orc_counters(self.h, _P(c))
        return c

    def measure(self):
        m = np.zeros(abi.NMEAS)
        self.lib.orc_measure(self.h, _P(m))
        return m

    def measure_local(self):
        out = np.zeros((self.p.sites(), 2))
        self.lib.orc_measure_local(self.h, _P(out))
        return out

    def measure_z(self):
        zd = ctypes.c_int()
        out = np.zeros((max(self.p.L[:3]), 4))
        self.lib.orc_measure_z(self.h, ctypes.byref(zd), _P(out))
        return zd.value, out[: self.p.L[zd.value]]

    def muca_set(self, w):
        self.lib.orc_muca_set(self.h, ctypes.byref(w.struct))

    def muca_get(self, w):
        self.lib.orc_muca_get(self.h, ctypes.byref(w.struct))
        w.pull()

    def grad_flow(self, t_max, dt, meas_interval, maxrows=4096):
        rows = np.zeros((maxrows, 1 + abi.NMEAS))
        n = ctypes.c_int(0)
        self.lib.orc_grad_flow(self.h, t_max, dt, meas_interval, _P(rows), maxrows, ctypes.byref(n))
        return rows[: n.value].copy()


class WeightBuf:
    """Host-side multicanonical weight with numpy-backed arrays."""

    def __init__(self, bins, orderparam=abi.PHISQ, mode=abi.MUCA_READONLY, checks_per_sweep=1):
        n = bins + 2
        self.pos = np.zeros(n)
        self.W = np.zeros(n)
        self.slope = np.zeros(n)
        self.b = np.zeros(n)
        self.hits = np.zeros(n, np.int32)
        self.gsum = np.zeros(n, np.int64)
        self.nsum = np.zeros(n, np.int64)
        self.hgram = np.zeros(n)
        s = abi.Weight()
        s.bins = bins
        s.orderparam = orderparam
        s.mode = mode
        s.checks_per_sweep = checks_per_sweep
        s.do_acceptance = 1
        s.update_interval = 100 if mode != abi.MUCA_SLOW else 5000
        s.pos = self.pos.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        s.W = self.W.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        s.slope = self.slope.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        s.b = self.b.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        s.hits = self.hits.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        s.gsum = self.gsum.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        s.nsum = self.nsum.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        s.hgram = self.hgram.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        self.struct = s

    def pull(self):
        pass

    def linearize(self):
        """linearize_weight (multicanonical.c:337-346)."""
        bins = self.struct.bins
        self.slope[0] = 0
        self.slope[bins + 1] = 0
        self.b[0] = self.W[0]
        self.b[bins + 1] = self.W[bins + 1]
        for i in range(1, bins + 1):
            self.slope[i] = (self.W[i + 1] - self.W[i]) / (self.pos[i + 1] - self.pos[i])
            self.b[i] = self.W[i] - self.slope[i] * self.pos[i]

    def scalars(self):
        s = self.struct
        return dict(bins=s.bins, min=s.min, max=s.max, wrk_min=s.wrk_min, wrk_max=s.wrk_max, delta=s.delta,
                    last_max=s.last_max, muca_count=s.muca_count, update_interval=s.update_interval,
                    mode=s.mode, pv0=s.param_value[0], pv1=s.param_value[1])


# ---------------------------------------------------------------------------
# reference harness
# ---------------------------------------------------------------------------
REF_VARIANT = {abi.HIGGS1: "fund", abi.TRIPLET: "adj", abi.HIGGS1 | abi.SINGLET | abi.U1: "su2u1s",
               abi.HIGGS1 | abi.TRIPLET: "fundadj", abi.HIGGS2 | abi.U1: "higgs2", 0: "pure"}


def ref_available(variant="fund"):
    return os.path.exists(os.path.join(REF_DIR, f"libref_{variant}.so"))


_ALG = {abi.METROPOLIS: "metropolis", abi.HEATBATH: "heatbath", abi.OVERRELAX: "overrelax"}


def reference_config(p, workdir, muca=None, flow=None, iterations=10, interval=1, reset=1, n_thermalize=0,
                     latticefile="lattice", resultsfile="/dev/null", extra=None):
    """A reference config file (su2higgs config:1-156 keys) equivalent to p."""
    lines = [f"dim {p.dim}"] + [f"L{d + 1} {p.L[d]}" for d in range(p.dim)]
    kv = dict(
        reset=reset, iterations=iterations, n_thermalize=n_thermalize, interval=interval, checkpoint=100000,
        run_checks=0, resultsfile=resultsfile, latticefile=latticefile,
        betasu2=repr(p.betasu2), betau1=repr(p.betau1), r_u1=repr(p.r_u1),
        msq=repr(p.msq_phi), **{"lambda": repr(p.lambda_phi)},
        msq_phi2=repr(p.msq_phi2), m12sq_re=repr(p.m12sq_re), m12sq_im=repr(p.m12sq_im),
        lam2=repr(p.lam2), lam3=repr(p.lam3), lam4=repr(p.lam4), lam5_re=repr(p.lam5_re),
        lam5_im=repr(p.lam5_im), lam6_re=repr(p.lam6_re), lam6_im=repr(p.lam6_im), lam7_re=repr(p.lam7_re),
        lam7_im=repr(p.lam7_im),
        msq_triplet=repr(p.msq_triplet), b4=repr(p.b4), a2=repr(p.a2),
        msq_s=repr(p.msq_s), b1_s=repr(p.b1_s), b3_s=repr(p.b3_s), b4_s=repr(p.b4_s), a1_s=repr(p.a1_s),
        a2_s=repr(p.a2_s), phi0=0.2, sigma0=0.2, singlet0=0.2,
        algorithm_su2link=_ALG[p.algorithm_su2link], algorithm_u1link=_ALG[p.algorithm_u1link],
        algorithm_su2doublet=_ALG[p.algorithm_su2doublet], algorithm_su2triplet=_ALG[p.algorithm_su2triplet],
        algorithm_singlet=_ALG[p.algorithm_singlet],
        scalar_sweeps=p.scalar_sweeps, update_singlet=p.update_singlet, update_doublet=p.update_su2doublet,
        update_triplet=p.update_su2triplet, update_links=p.update_links,
        multicanonical=0, measure_local=0, do_flow=0, flow_meas_interval=10, flow_dt=0.05, flow_interval=1000,
        flow_t_max=10, do_correlators=0, correlator_interval=1000, blocks=0,
    )
    if muca is not None:
        kv.update(multicanonical=1, **muca)
    if flow is not None:
        kv.update(do_flow=1, **flow)
    if extra:
        kv.update(extra)
    lines += [f"{k} {v}" for k, v in kv.items()]
    path = os.path.join(workdir, "config")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    return path


class Ref:
    """The reference itself (compiled from its sources) behind the harness."""

    _libs = {}

    def __init__(self, p, workdir=None, muca=None, flow=None, variant=None):
        variant = variant or REF_VARIANT[p.content & ~abi.GRADFLOW]
        path = os.path.join(REF_DIR, f"libref_{variant}.so")
        # each instance needs fresh globals: load a private copy of the library
        self.workdir = workdir or tempfile.mkdtemp(prefix="su2ref_")
        priv = os.path.join(self.workdir, f"libref_{variant}.so")
        if not os.path.exists(priv):
            with open(path, "rb") as src, open(priv, "wb") as dst:
                dst.write(src.read())
        lib = ctypes.CDLL(priv)
        lib.ref_sites.restype = ctypes.c_long
        lib.ref_evensites.restype = ctypes.c_long
        lib.ref_set_rng.argtypes = [ctypes.c_ulonglong, ctypes.c_uint, ctypes.c_uint]
        lib.ref_site_update.argtypes = [ctypes.c_int, ctypes.c_long, ctypes.c_int, ctypes.c_uint]
        for name in ("ref_localact_su2link", "ref_localact_u1link"):
            if hasattr(lib, name):
                getattr(lib, name).restype = ctypes.c_double
                getattr(lib, name).argtypes = [ctypes.c_long, ctypes.c_int]
        for name in ("ref_local_su2wilson", "ref_action_local", "ref_higgspotential", "ref_local_u1wilson",
                     "ref_localact_triplet", "ref_covariant_triplet", "ref_magcharge_cube", "ref_localact_singlet"):
            if hasattr(lib, name):
                getattr(lib, name).restype = ctypes.c_double
                getattr(lib, name).argtypes = [ctypes.c_long]
        for name in ("ref_localact_doublet", "ref_covariant_doublet"):
            if hasattr(lib, name):
                getattr(lib, name).restype = ctypes.c_double
                getattr(lib, name).argtypes = [ctypes.c_long, ctypes.c_int]
        if hasattr(lib, "ref_alpha_proj"):
            lib.ref_alpha_proj.restype = ctypes.c_double
            lib.ref_alpha_proj.argtypes = [ctypes.c_long, ctypes.c_int, ctypes.c_int]
        for name in ("ref_link_staple", "ref_wilson_staple", "ref_staple_doublet"):
            if hasattr(lib, name):
                getattr(lib, name).argtypes = [ctypes.c_long, ctypes.c_int, ctypes.c_void_p]
        lib.ref_or_proposal.argtypes = [ctypes.c_int, ctypes.c_long, ctypes.c_int, ctypes.c_void_p]
        lib.ref_polysolve3.restype = ctypes.c_double
        lib.ref_polysolve3.argtypes = [ctypes.c_double] * 4
        lib.ref_calc_orderparam.restype = ctypes.c_double
        lib.ref_calc_orderparam.argtypes = [ctypes.c_int]
        lib.ref_get_weight.restype = ctypes.c_double
        lib.ref_get_weight.argtypes = [ctypes.c_double]
        lib.ref_whichbin.argtypes = [ctypes.c_double]
        if hasattr(lib, "ref_flow_step"):
            lib.ref_flow_step.argtypes = [ctypes.c_double]
            lib.ref_grad_flow.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_void_p,
                                          ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        if hasattr(lib, "ref_correlators"):
            lib.ref_correlators.argtypes = [ctypes.c_int, ctypes.c_void_p]
        if hasattr(lib, "ref_blocked_level"):
            lib.ref_blocked_level.restype = ctypes.c_long
            lib.ref_blocked_level.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 5
        self.lib = lib
        self.p = p
        cfg = reference_config(p, self.workdir, muca=muca, flow=flow)
        cwd = os.getcwd()
        os.chdir(self.workdir)
        try:
            lib.ref_setup(cfg.encode())
        finally:
            os.chdir(cwd)
        self.V = lib.ref_sites()

    def longest_dir(self):
        return self.lib.ref_longest_dir()

    def correlators(self, dir):
        """measure_correlators() values (correlation.c:350-398), full precision:
        rows d < L[dir]/2 of (Higgs, Sigma^2, photon (1,0), (2,0), (1,1), (2,1)
        re/im)."""
        out = np.zeros((self.p.L[dir] // 2 + 1, 10))
        n = self.lib.ref_correlators(dir, _P(out))
        return out[:n].copy()

    def block_setup(self, levels):
        return self.lib.ref_block_setup(levels)

    def blocked_level(self, k, dir):
        """Smear level k (0 = the lattice itself), move it onto blocked level
        k+1 and measure its correlators (correlation.c:404-432); returns the
        correlator rows, the blocked links / triplet in the blocked lattice's
        storage order, its coordinates and sides."""
        V, D = self.V, self.p.dim
        corr = np.zeros((self.p.L[dir] // 2 + 1, 10))
        link, trip = np.zeros(V * D * 4), np.zeros(V * 3)
        coords, Lb = np.zeros(V * D, np.int64), np.zeros(4, np.int32)
        n = self.lib.ref_blocked_level(k, dir, _P(corr), _P(link), _P(trip), _P(coords), _P(Lb))
        assert n > 0
        return dict(corr=corr[: self.p.L[dir] // 2].copy(), link=link[: n * D * 4].reshape(n, D, 4).copy(),
                    trip=trip[: n * 3].reshape(n, 3).copy(), coords=coords[: n * D].reshape(n, D).copy(),
                    L=Lb[:D].copy())

    def tables(self):
        V, D = self.V, self.p.dim
        nx, pv, co = (np.zeros(V * D, np.int64) for _ in range(3))
        par = np.zeros(V, np.int32)
        self.lib.ref_tables(_P(nx), _P(pv), _P(co), _P(par))
        return nx.reshape(V, D), pv.reshape(V, D), co.reshape(V, D), par

    def put(self, f):
        self.lib.ref_put_fields(*f.ptrs())

    def get(self):
        f = Fields(self.p)
        self.lib.ref_get_fields(*f.ptrs())
        return f

    def set_rng(self, seed, sweep, chain=0):
        self.lib.ref_set_rng(seed, sweep, chain)

    def update(self):
        cwd = os.getcwd()
        os.chdir(self.workdir)
        try:
            return self.lib.ref_update()
        finally:
            os.chdir(cwd)

    def counters(self):
        c = np.zeros(abi.NCOUNTERS, np.int64)
        self.lib.ref_counters(_P(c))
        return c

    def measure_raw(self):
        out = np.zeros(64)
        row = ctypes.create_string_buffer(4096)
        n = self.lib.ref_measure_sums(_P(out), row, 4096)
        return out[:n].copy(), row.value.decode()

    def measure(self):
        raw, _ = self.measure_raw()
        return ref_sums_to_layout(self.p, raw)

    def muca_init(self):
        cwd = os.getcwd()
        os.chdir(self.workdir)
        try:
            return self.lib.ref_muca_init()
        finally:
            os.chdir(cwd)

    def muca_state(self):
        sc = np.zeros(12)
        self.lib.ref_muca_scalars(_P(sc))
        bins = int(sc[0])
        n = bins + 2
        pos, W, slope, b = (np.zeros(n) for _ in range(4))
        hits = np.zeros(n, np.int32)
        self.lib.ref_muca_arrays(_P(pos), _P(W), _P(slope), _P(b), _P(hits))
        pv = np.zeros(2)
        self.lib.ref_muca_values(_P(pv))
        gsum, nsum, hgram = np.zeros(n, np.int64), np.zeros(n, np.int64), np.zeros(n)
        self.lib.ref_muca_slow_arrays(_P(gsum), _P(nsum), _P(hgram))
        return dict(bins=bins, min=sc[1], max=sc[2], wrk_min=sc[3], wrk_max=sc[4], delta=sc[5],
                    last_max=int(sc[6]), muca_count=int(sc[7]), update_interval=int(sc[8]), mode=int(sc[9]),
                    checks_per_sweep=int(sc[10]), orderparam=int(sc[11]), pos=pos, W=W, slope=slope, b=b,
                    hits=hits, param_value=pv, gsum=gsum, nsum=nsum, hgram=hgram)

    def muca_set_update_interval(self, n):
        self.lib.ref_muca_set_update_interval(n)

    def grad_flow(self, t_max, dt, flow_id=1, maxrows=2048):
        per = 64
        out = np.zeros(maxrows * per)
        n = ctypes.c_int(0)
        cwd = os.getcwd()
        os.chdir(self.workdir)
        try:
            k = self.lib.ref_grad_flow(t_max, dt, flow_id, _P(out), maxrows, ctypes.byref(n))
        finally:
            os.chdir(cwd)
        return out[: n.value * k].reshape(n.value, k)


def weight_from_state(st):
    """WeightBuf holding a weight state dict (as returned by Ref.muca_state)."""
    w = WeightBuf(st["bins"], orderparam=st["orderparam"], mode=st["mode"],
                  checks_per_sweep=st["checks_per_sweep"])
    for k in ("pos", "W", "slope", "b", "hits"):
        getattr(w, k)[:] = st[k]
    s = w.struct
    s.min, s.max, s.wrk_min, s.wrk_max, s.delta = st["min"], st["max"], st["wrk_min"], st["wrk_max"], st["delta"]
    s.last_max, s.muca_count, s.update_interval = st["last_max"], st["muca_count"], st["update_interval"]
    s.param_value[0], s.param_value[1] = st["param_value"]
    return w


def ref_sums_to_layout(p, raw):
    """Map the reduce_sum() capture order of measure() (measure.c:191-233) to
    the fixed SU2GPU_M_* layout."""
    m = np.zeros(abi.NMEAS)
    k = 0

    def take():
        nonlocal k
        v = raw[k]
        k += 1
        return v

    m[abi.M_ACTION] = take()
    m[abi.M_WILSON] = take()
    if p.content & abi.U1:
        m[abi.M_U1WILSON] = take()
    nh = p.nhiggs()
    for h in range(nh):
        m[abi.M_COV_PHI + 3 * h] = take()
        m[abi.M_PHI2 + 3 * h] = take()
        m[abi.M_PHI4 + 3 * h] = take()
    if nh == 2:
        m[abi.M_PHI12_RE] = take()
        m[abi.M_PHI12_IM] = take()
    if p.content & abi.TRIPLET:
        m[abi.M_HOP_SIGMA] = take()
        m[abi.M_SIGMA2] = take()
        m[abi.M_SIGMA4] = take()
        m[abi.M_MAGCHARGE] = take()
        m[abi.M_MAGCHARGE_ABS] = take()
        if nh > 0:
            m[abi.M_PHI2SIGMA2] = take()
    if p.content & abi.SINGLET:
        m[abi.M_S_COV] = take()
        for idx in (abi.M_S1, abi.M_S2, abi.M_S3, abi.M_S4):
            m[idx] = take()
        if nh == 1:
            m[abi.M_SPHI2] = take()
            m[abi.M_S2PHI2] = take()
    assert k == len(raw), (k, len(raw))
    return m


def layout_digest(nx, pv, co, par):
    """SHA-256 of the layout tables (next, prev, coords as little-endian
    int64 [V][D], then parity as int32 [V])."""
    import hashlib
    h = hashlib.sha256()
    for a in (nx, pv, co):
        h.update(np.ascontiguousarray(a, dtype="<i8").tobytes())
    h.update(np.ascontiguousarray(par, dtype="<i4").tobytes())
    return h.hexdigest()


def rel_err(a, b, floor=1e-300):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.maximum(np.maximum(np.abs(a), np.abs(b)), floor)
    return float(np.max(np.abs(a - b) / den)) if a.size else 0.0


def oracle_sweep_order(seed, chain, sweep, update_links=1, scalar_sweeps=4, D=3):
    """The oracle's pass order of `sweep` in random_sweeps mode."""
    lib = oracle_lib()
    d = np.zeros((max(update_links, 1), 2 * D), np.int32)
    q = np.zeros((max(update_links, 1), 2 * D), np.int32)
    f = np.zeros(scalar_sweeps + 1, np.int32)
    lib.orc_sweep_order(seed, chain, sweep, D, update_links, scalar_sweeps, _P(d), _P(q), _P(f))
    return d[:update_links], q[:update_links], f
