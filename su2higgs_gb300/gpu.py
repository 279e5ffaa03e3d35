"""Python binding of libsu2gpu (include/su2gpu.h) through ctypes.

`Lattice` mirrors the reference's per-lattice entry points: update_lattice()
(update.c:270), measure() sums (measure.c:71), grad_flow() (gradflow.c:46),
calc_orderparam() (multicanonical.c:709) and the field transfer that stands in
for load_lattice()/save_lattice() (checkpoint.c:84-214).  Host field arrays are
FP64, array-of-structures, in the reference's EVEN-first site order.

There is no CPU fallback: every call goes to the CUDA library, and a missing
library or device raises.
"""
import ctypes
import os

import numpy as np

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libsu2gpu.so")

_lib = None


class SU2GPUError(RuntimeError):
    pass


def lib():
    """The loaded libsu2gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise SU2GPUError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(LIB_PATH)
        vp, i32, u32, u64, i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int64
        dp = ctypes.POINTER(ctypes.c_double)
        L.su2gpu_last_error.restype = ctypes.c_char_p
        L.su2gpu_create.argtypes = [ctypes.POINTER(abi.Params), ctypes.POINTER(vp)]
        L.su2gpu_destroy.argtypes = [vp]
        L.su2gpu_footprint_bytes.restype = i64
        L.su2gpu_footprint_bytes.argtypes = [ctypes.POINTER(abi.Params)]
        L.su2gpu_layout_tables.argtypes = [vp, vp, vp, vp, vp]
        L.su2gpu_site_values.argtypes = [vp, i32, vp]
        L.su2gpu_upload_fields.argtypes = [vp] + [vp] * 6
        L.su2gpu_download_fields.argtypes = [vp] + [vp] * 6
        L.su2gpu_set_seed.argtypes = [vp, u64, u32]
        L.su2gpu_update_lattice.argtypes = [vp, u32]
        L.su2gpu_run_sweeps.argtypes = [vp, u32, i32, i32]
        L.su2gpu_get_counters.argtypes = [vp, vp]
        L.su2gpu_reset_counters.argtypes = [vp]
        L.su2gpu_measure.argtypes = [vp, vp]
        L.su2gpu_muca_set.argtypes = [vp, ctypes.POINTER(abi.Weight)]
        L.su2gpu_muca_get.argtypes = [vp, ctypes.POINTER(abi.Weight)]
        L.su2gpu_muca_weight_updates.argtypes = [vp, ctypes.POINTER(i32)]
        L.su2gpu_calc_orderparam.argtypes = [vp, i32, dp]
        L.su2gpu_muca_init_last_max.argtypes = [vp]
        L.su2gpu_grad_flow.argtypes = [vp, ctypes.c_double, ctypes.c_double, i32, vp, i32, ctypes.POINTER(i32)]
        L.su2gpu_grad_flow_local.argtypes = [vp, ctypes.c_double, ctypes.c_double, i32, vp, i32, ctypes.POINTER(i32),
                                             vp, i32]
        L.su2gpu_measure_local.argtypes = [vp, vp]
        L.su2gpu_measure_z.argtypes = [vp, ctypes.POINTER(i32), vp]
        L.su2gpu_update_lattice_host.argtypes = [vp, u32] + [vp] * 6
        L.su2gpu_stream_uniform.restype = ctypes.c_double
        L.su2gpu_stream_uniform.argtypes = [u64, u32, u32, u32, u32, u32]
        L.su2gpu_device_info.argtypes = [ctypes.POINTER(ctypes.c_int)] * 3 + [ctypes.POINTER(i64)]
        L.su2gpu_set_stream.argtypes = [vp, vp]
        L.su2gpu_set_random_sweeps.argtypes = [vp, i32]
        L.su2gpu_clone.argtypes = [vp, u64, u32, ctypes.POINTER(vp)]
        L.su2gpu_measure_correlators.argtypes = [vp, i32, vp]
        L.su2gpu_measure_blocked_correlators.argtypes = [vp, i32, vp, i32, vp, ctypes.POINTER(i32)]
        L.su2gpu_blocked_fields.argtypes = [vp, vp, i32, vp, vp, vp]
        L.su2gpu_copy_fields.argtypes = [vp, vp]
        L.su2gpu_sweep_order.argtypes = [u64, u32, u32, i32, i32, vp, vp, vp]
        L.su2gpu_enqueue_sweeps.argtypes = [vp, u32, i32, i32]
        L.su2gpu_enqueue_measure.argtypes = [vp, vp]
        L.su2gpu_launches_per_sweep.argtypes = [vp, ctypes.POINTER(i32)]
        L.su2gpu_profile_sweep.argtypes = [vp, u32, i32, vp, vp, ctypes.POINTER(i32)]
        L.su2gpu_host_register.argtypes = [vp, i64]
        L.su2gpu_host_unregister.argtypes = [vp]
        L.su2gpu_run_halfsweep.argtypes = [vp, i32, i32, i32, u32, u32]
        L.su2gpu_autotune.argtypes = [vp, vp, vp]
        L.su2gpu_set_variants.argtypes = [vp, vp]
        P = ctypes.POINTER(abi.Params)
        L.su2gpu_pool_chain_bytes.restype = i64
        L.su2gpu_pool_chain_bytes.argtypes = [P]
        L.su2gpu_pool_create.argtypes = [P, i64, i32, ctypes.POINTER(vp)]
        L.su2gpu_pool_destroy.argtypes = [vp]
        L.su2gpu_pool_add.argtypes = [vp, P, u64, u32, ctypes.POINTER(i32)]
        L.su2gpu_pool_remove.argtypes = [vp, i32]
        L.su2gpu_pool_info.argtypes = [vp, ctypes.POINTER(i32)] + [ctypes.POINTER(i64)] * 3
        L.su2gpu_pool_active.argtypes = [vp, vp, i32, ctypes.POINTER(i32)]
        L.su2gpu_pool_upload.argtypes = [vp, i32] + [vp] * 6
        L.su2gpu_pool_download.argtypes = [vp, i32] + [vp] * 6
        L.su2gpu_pool_set_sweep.argtypes = [vp, i32, u32]
        L.su2gpu_pool_run.argtypes = [vp, i32, i32]
        L.su2gpu_pool_measure.argtypes = [vp, vp, i32, ctypes.POINTER(i32)]
        L.su2gpu_pool_counters.argtypes = [vp, i32, vp]
        L.su2gpu_pool_autotune.argtypes = [vp, vp, vp]
        L.su2gpu_pool_set_variants.argtypes = [vp, vp]
        L.su2gpu_pool_extract.argtypes = [vp, i32, ctypes.POINTER(vp)]
        L.su2gpu_pool_upload_many.argtypes = [vp, i32, vp, vp]
        L.su2gpu_pool_download_many.argtypes = [vp, i32, vp, vp]
        L.su2gpu_pool_cycle.argtypes = [vp, i32, vp, vp, i32, i32, vp, vp]
        L.su2gpu_pool_enqueue.argtypes = [vp, i32, i32]
        L.su2gpu_pool_set_persistent.argtypes = [vp, i32]
        L.su2gpu_pool_get_persist_tiles.argtypes = [vp, ctypes.POINTER(i32)]
        L.su2gpu_pool_set_persist_shape.argtypes = [vp, i32]
        L.su2gpu_pool_get_persist_shape.argtypes = [vp, ctypes.POINTER(i32), ctypes.POINTER(i32), ctypes.POINTER(i32)]
        L.su2gpu_pool_get_persistent.argtypes = [vp, ctypes.POINTER(i32)]
        L.su2gpu_pool_set_sweep_groups.argtypes = [vp, i32, i32]
        L.su2gpu_pool_get_sweep_groups.argtypes = [vp, ctypes.POINTER(i32), ctypes.POINTER(i32)]
        L.su2gpu_pool_check_wait_timeout.argtypes = [vp, i32, ctypes.POINTER(i32)]
        L.su2gpu_pool_raise_error.argtypes = [vp, i32]
        L.su2gpu_pool_muca_set.argtypes = [vp, i32, ctypes.POINTER(abi.Weight)]
        L.su2gpu_pool_muca_get.argtypes = [vp, i32, ctypes.POINTER(abi.Weight)]
        L.su2gpu_pool_calc_orderparam.argtypes = [vp, i32, i32, ctypes.POINTER(ctypes.c_double)]
        L.su2gpu_pool_enqueue_measure.argtypes = [vp, vp, i32, ctypes.POINTER(i32)]
        L.su2gpu_pool_set_stream.argtypes = [vp, vp]
        L.su2gpu_pool_launches_per_sweep.argtypes = [vp, ctypes.POINTER(i32)]
        L.su2gpu_pool_profile_sweep.argtypes = [vp, i32, vp, vp, ctypes.POINTER(i32)]
        L.su2gpu_pool_grad_flow.argtypes = [vp, i32, ctypes.c_double, ctypes.c_double, i32, vp, i32,
                                            ctypes.POINTER(i32)]
        _lib = L
    return _lib


def check(rc):
    if rc != abi.OK:
        raise SU2GPUError(f"libsu2gpu error {rc}: {lib().su2gpu_last_error().decode()}")
    return rc


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


FIELD_NAMES = ("link", "u1", "d0", "d1", "trip", "sing")


class Lattice:
    """One device-resident chain (a su2gpu context)."""

    def __init__(self, params, seed=0, chain=0, _handle=None):
        self.params = params
        self.V = params.sites()
        if _handle is not None:  # a context made by another entry point (Pool.extract)
            self._h = _handle
            return
        self._h = ctypes.c_void_p()
        check(lib().su2gpu_create(ctypes.byref(params), ctypes.byref(self._h)))
        check(lib().su2gpu_set_seed(self._h, seed, chain))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().su2gpu_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def shapes(self):
        p, V = self.params, self.V
        nh = p.nhiggs()
        return {
            "link": (V, 3, 4),
            "u1": (V, 3) if p.content & abi.U1 else None,
            "d0": (V, 4) if nh > 0 else None,
            "d1": (V, 4) if nh > 1 else None,
            "trip": (V, 3) if p.content & abi.TRIPLET else None,
            "sing": (V,) if p.content & abi.SINGLET else None,
        }

    def upload(self, **fields):
        arrs = []
        for n in FIELD_NAMES:
            a = fields.get(n)
            arrs.append(None if a is None else np.ascontiguousarray(a, dtype=np.float64))
        check(lib().su2gpu_upload_fields(self._h, *[_p(a) for a in arrs]))

    def download(self):
        out = {}
        for n, shp in self.shapes().items():
            out[n] = None if shp is None else np.zeros(shp)
        check(lib().su2gpu_download_fields(self._h, *[_p(out[n]) for n in FIELD_NAMES]))
        return out

    def set_seed(self, seed, chain=0):
        check(lib().su2gpu_set_seed(self._h, seed, chain))

    def update_lattice(self, sweep):
        check(lib().su2gpu_update_lattice(self._h, sweep))

    def clone(self, seed, chain=0):
        """A new chain with a device copy of this one's fields."""
        h = ctypes.c_void_p()
        check(lib().su2gpu_clone(self._h, seed, chain, ctypes.byref(h)))
        return Lattice(self.params, _handle=h)

    def copy_fields_from(self, other):
        """Device copy of `other`'s fields into this chain (same lattice,
        content and precision)."""
        check(lib().su2gpu_copy_fields(self._h, other._h))

    def set_random_sweeps(self, on=True):
        """The reference's random_sweeps mode: the pass order of every sweep
        drawn from the order stream (sweep_order)."""
        check(lib().su2gpu_set_random_sweeps(self._h, 1 if on else 0))

    def run_sweeps(self, first_sweep, n, graph=True):
        check(lib().su2gpu_run_sweeps(self._h, first_sweep, n, 1 if graph else 0))

    def autotune(self):
        """Pick the fastest launch shape per update kernel kind; returns
        (choices, mean launch ms) for link, U(1), doublet, triplet, singlet."""
        ch = np.zeros(5, np.int32)
        ms = np.zeros(5, np.float32)
        check(lib().su2gpu_autotune(self._h, _p(ch), _p(ms)))
        return ch, ms

    def set_variants(self, choices):
        ch = np.ascontiguousarray(choices, dtype=np.int32)
        check(lib().su2gpu_set_variants(self._h, _p(ch)))

    def run_halfsweep(self, kind, parity, sub, pass_, sweep):
        """One half-sweep (kind 0 links, 1 U(1), 2/3 doublet OR|Metropolis,
        4/5 triplet, 6/7 singlet; see su2gpu_run_halfsweep)."""
        check(lib().su2gpu_run_halfsweep(self._h, kind, parity, sub, pass_, sweep))

    def counters(self):
        c = np.zeros(abi.NCOUNTERS, np.int64)
        check(lib().su2gpu_get_counters(self._h, _p(c)))
        return c

    def reset_counters(self):
        check(lib().su2gpu_reset_counters(self._h))

    def measure(self):
        m = np.zeros(abi.NMEAS)
        check(lib().su2gpu_measure(self._h, _p(m)))
        return m

    SITE_VALUES = {"link_staple": (1, (3, 4)), "wilson_staple": (2, (3, 4)), "localact_su2link": (3, (3,)),
                   "localact_u1link": (4, (3,)), "staple_doublet": (5, (4,)), "localact_doublet": (6, ()),
                   "localact_singlet": (7, ()), "or_doublet": (8, (4,)), "or_doublet1": (9, (4,)),
                   "or_triplet": (10, (3,)), "or_singlet": (11, ())}

    def site_values(self, name):
        """Per-site values of a deterministic kernel (su2gpu_site_values),
        named as the keys of SITE_VALUES; shape (V,) + the value's shape."""
        what, shape = self.SITE_VALUES[name]
        out = np.zeros((self.V,) + shape)
        check(lib().su2gpu_site_values(self._h, what, _p(out)))
        return out

    def layout_tables(self):
        V = self.V
        nx, pv, co = (np.zeros(V * 3, np.int64) for _ in range(3))
        par = np.zeros(V, np.int32)
        check(lib().su2gpu_layout_tables(self._h, _p(nx), _p(pv), _p(co), _p(par)))
        return nx.reshape(V, 3), pv.reshape(V, 3), co.reshape(V, 3), par

    def muca_set(self, weight_struct):
        check(lib().su2gpu_muca_set(self._h, ctypes.byref(weight_struct)))

    def muca_get(self, weight_struct):
        check(lib().su2gpu_muca_get(self._h, ctypes.byref(weight_struct)))

    def muca_weight_updates(self):
        n = ctypes.c_int32(0)
        check(lib().su2gpu_muca_weight_updates(self._h, ctypes.byref(n)))
        return n.value

    def calc_orderparam(self, parity):
        v = ctypes.c_double(0)
        check(lib().su2gpu_calc_orderparam(self._h, parity, ctypes.byref(v)))
        return v.value

    def muca_init_last_max(self):
        check(lib().su2gpu_muca_init_last_max(self._h))

    def grad_flow(self, t_max, dt, meas_interval, maxrows=None):
        if maxrows is None:
            maxrows = int(t_max / dt) // meas_interval + 4
        rows = np.zeros((maxrows, 1 + abi.NMEAS))
        n = ctypes.c_int32(0)
        check(lib().su2gpu_grad_flow(self._h, t_max, dt, meas_interval, _p(rows), maxrows, ctypes.byref(n)))
        return rows[: n.value].copy()

    def measure_local(self):
        """measure_local (measure.c:368): per site in storage order,
        (Tr Sigma^2, magnetic charge in units of 2 pi sqrt(beta))."""
        out = np.zeros((self.V, 2))
        check(lib().su2gpu_measure_local(self._h, _p(out)))
        return out

    def measure_z(self):
        """measure_along_z (z_coord.c:206): (z direction, plane sums of
        phi^2, Tr Sigma^2, S, S^2 for every z)."""
        zd = ctypes.c_int32()
        out = np.zeros((max(self.params.L[:3]), 4))
        check(lib().su2gpu_measure_z(self._h, ctypes.byref(zd), _p(out)))
        return zd.value, out[: self.params.L[zd.value]].copy()

    def longest_dir(self):
        """The direction the reference measures correlators along
        (make_misc_tables, layout.c:773-777): the longest, ties to the last."""
        L = self.params.L
        ld = 2
        for d in (2, 1, 0):
            if L[d] > L[ld]:
                ld = d
        return ld

    def measure_correlators(self, dir=None):
        """measure_correlators (correlation.c:350-398): rows d < L[dir]/2 of
        abi.NCORR values."""
        dir = self.longest_dir() if dir is None else dir
        out = np.zeros((self.params.L[dir] // 2, abi.NCORR))
        check(lib().su2gpu_measure_correlators(self._h, dir, _p(out)))
        return out

    def _block_sides(self, block_dir, levels):
        sides = [tuple(self.params.L[:3])]
        for _ in range(levels):
            sides.append(tuple(n // 2 if b else n for n, b in zip(sides[-1], block_dir)))
        return sides

    def measure_blocked_correlators(self, block_dir, levels, dir=None):
        """Correlators of blocking levels 1..levels (as many as the sides
        allow): a list with one (L_k[dir]/2, NCORR) array per level made."""
        dir = self.longest_dir() if dir is None else dir
        bd = np.ascontiguousarray(block_dir, dtype=np.int32)
        sides = self._block_sides(bd, levels)
        out = np.zeros((sum(s[dir] // 2 for s in sides[1:]) + 1, abi.NCORR))
        done = ctypes.c_int32()
        check(lib().su2gpu_measure_blocked_correlators(self._h, dir, _p(bd), levels, _p(out), ctypes.byref(done)))
        res, r = [], 0
        for s in sides[1: 1 + done.value]:
            res.append(out[r: r + s[dir] // 2].copy())
            r += s[dir] // 2
        return res

    def blocked_fields(self, block_dir, level):
        """Fields of blocking level `level` in its lexicographic order:
        (sides, links (n, 3, 4), triplet (n, 3) or None)."""
        bd = np.ascontiguousarray(block_dir, dtype=np.int32)
        s = self._block_sides(bd, level)[-1]
        n = s[0] * s[1] * s[2]
        Lb = np.zeros(3, np.int32)
        link = np.zeros((n, 3, 4))
        trip = np.zeros((n, 3)) if self.params.content & abi.TRIPLET else None
        check(lib().su2gpu_blocked_fields(self._h, _p(bd), level, _p(Lb), _p(link), _p(trip)))
        assert tuple(Lb) == s
        return s, link, trip

    def grad_flow_local(self, t_max, dt, meas_interval, maxrows=None):
        """grad_flow plus measure_local of the flowed fields at every
        measurement: (rows, array of shape (rows, V, 2))."""
        if maxrows is None:
            maxrows = int(t_max / dt) // meas_interval + 4
        rows = np.zeros((maxrows, 1 + abi.NMEAS))
        local = np.zeros((maxrows, self.V, 2))
        n = ctypes.c_int32(0)
        check(lib().su2gpu_grad_flow_local(self._h, t_max, dt, meas_interval, _p(rows), maxrows, ctypes.byref(n),
                                           _p(local), maxrows))
        return rows[: n.value].copy(), local[: n.value].copy()

    def set_stream(self, stream_ptr):
        """Run on a caller's CUDA stream (an int cudaStream_t, e.g.
        torch.cuda.current_stream().cuda_stream); 0/None = own stream."""
        check(lib().su2gpu_set_stream(self._h, ctypes.c_void_p(stream_ptr or None)))

    def enqueue_sweeps(self, first_sweep, n, graph=True):
        check(lib().su2gpu_enqueue_sweeps(self._h, first_sweep, n, 1 if graph else 0))

    def enqueue_measure(self, device_ptr):
        check(lib().su2gpu_enqueue_measure(self._h, ctypes.c_void_p(device_ptr)))

    def launches_per_sweep(self):
        n = ctypes.c_int32(0)
        check(lib().su2gpu_launches_per_sweep(self._h, ctypes.byref(n)))
        return n.value

    def profile_sweep(self, sweep, maxp=4096):
        kinds = np.zeros(maxp, np.int32)
        ms = np.zeros(maxp, np.float32)
        n = ctypes.c_int32(0)
        check(lib().su2gpu_profile_sweep(self._h, sweep, maxp, _p(kinds), _p(ms), ctypes.byref(n)))
        return kinds[: n.value].copy(), ms[: n.value].astype(np.float64)

    def update_lattice_host(self, sweep, fields):
        """Drop-in update_lattice(): host arrays in, updated host arrays out."""
        arrs = [fields.get(n) for n in FIELD_NAMES]
        check(lib().su2gpu_update_lattice_host(self._h, sweep, *[_p(a) for a in arrs]))


def stream_uniform(seed, site, pass_, draw, sweep, chain=0):
    """The uniform the kernels draw (host evaluation of the Philox stream)."""
    return lib().su2gpu_stream_uniform(seed, site, pass_, draw, sweep, chain)


def sweep_order(seed, chain, sweep, update_links=1, scalar_sweeps=4):
    """Pass order of `sweep` in random_sweeps mode: (link_dirs, link_pars)
    as (update_links, 6) arrays and the parity each scalar sweep starts
    with (scalar_sweeps + 1 entries, 0 EVEN)."""
    d = np.zeros((max(update_links, 1), 6), np.int32)
    q = np.zeros((max(update_links, 1), 6), np.int32)
    f = np.zeros(scalar_sweeps + 1, np.int32)
    check(lib().su2gpu_sweep_order(seed, chain, sweep, update_links, scalar_sweeps, _p(d), _p(q), _p(f)))
    return d[:update_links], q[:update_links], f


def host_register(arr):
    """Page-lock a numpy array for the host-buffer entry points."""
    check(lib().su2gpu_host_register(_p(arr), arr.nbytes))


def host_unregister(arr):
    check(lib().su2gpu_host_unregister(_p(arr)))


def device_info():
    sm, ma, mi = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    fr = ctypes.c_int64()
    check(lib().su2gpu_device_info(ctypes.byref(sm), ctypes.byref(ma), ctypes.byref(mi), ctypes.byref(fr)))
    return dict(sm_count=sm.value, cc=(ma.value, mi.value), free_bytes=fr.value)


def _shapes(p):
    V, nh = p.sites(), p.nhiggs()
    return {
        "link": (V, 3, 4),
        "u1": (V, 3) if p.content & abi.U1 else None,
        "d0": (V, 4) if nh > 0 else None,
        "d1": (V, 4) if nh > 1 else None,
        "trip": (V, 3) if p.content & abi.TRIPLET else None,
        "sing": (V,) if p.content & abi.SINGLET else None,
    }


class CapacityError(SU2GPUError):
    """The pool's arena or slot table cannot take the chain."""


class Pool:
    """Many independent chains of one content / precision / update recipe in
    one device arena (a su2gpu pool); every half-sweep is one launch over all
    chains.  A chain follows the trajectory of a `Lattice` with the same
    parameters, seed and chain id."""

    def __init__(self, recipe, arena_bytes, max_chains=1024):
        self.recipe = recipe
        self._h = ctypes.c_void_p()
        self._params = {}
        check(lib().su2gpu_pool_create(ctypes.byref(recipe), int(arena_bytes), int(max_chains),
                                       ctypes.byref(self._h)))

    def close(self):
        self.__dict__.pop("_tcache", None)
        if getattr(self, "_h", None) and self._h.value:
            lib().su2gpu_pool_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def chain_bytes(params):
        return int(lib().su2gpu_pool_chain_bytes(ctypes.byref(params)))

    def add(self, params, seed=0, chain=0):
        """Admit a chain; returns its slot.  Raises CapacityError when the
        arena or the slot table is full."""
        s = ctypes.c_int32()
        rc = lib().su2gpu_pool_add(self._h, ctypes.byref(params), seed, chain, ctypes.byref(s))
        if rc == abi.ERR_CAPACITY:
            raise CapacityError(lib().su2gpu_last_error().decode())
        check(rc)
        self._params[s.value] = params
        return s.value

    def remove(self, slot):
        check(lib().su2gpu_pool_remove(self._h, slot))
        self._params.pop(slot, None)

    def info(self):
        n, u, f, b = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        check(lib().su2gpu_pool_info(self._h, ctypes.byref(n), ctypes.byref(u), ctypes.byref(f), ctypes.byref(b)))
        return {"chains": n.value, "used_bytes": u.value, "free_bytes": f.value, "largest_free": b.value}

    def active(self):
        n = ctypes.c_int32()
        check(lib().su2gpu_pool_active(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros(max(n.value, 1), dtype=np.int32)
        check(lib().su2gpu_pool_active(self._h, _p(out), n.value, ctypes.byref(n)))
        return out[:n.value]

    def upload(self, slot, **fields):
        arrs = [None if fields.get(n) is None else np.ascontiguousarray(fields[n], dtype=np.float64)
                for n in FIELD_NAMES]
        check(lib().su2gpu_pool_upload(self._h, slot, *[_p(a) for a in arrs]))

    def download(self, slot, out=None):
        """The chain's FP64 host fields; `out` (a dict of C-contiguous float64
        arrays of the right shapes) receives them in place when given."""
        shapes = _shapes(self._params[slot])
        if out is None:
            out = {n: (None if shp is None else np.zeros(shp)) for n, shp in shapes.items()}
        for n, shp in shapes.items():
            a = out.get(n)
            if a is not None and (a.shape != shp or a.dtype != np.float64 or not a.flags.c_contiguous):
                raise ValueError(f"{n}: need a C-contiguous float64 array of shape {shp}")
        check(lib().su2gpu_pool_download(self._h, slot, *[_p(out.get(n)) for n in FIELD_NAMES]))
        return out

    @staticmethod
    def _tables(n, fields, keep):
        tables = (ctypes.c_void_p * 6)()
        for k, name in enumerate(FIELD_NAMES):
            arrs = [f.get(name) for f in fields]
            if all(a is None for a in arrs):
                continue
            t = (ctypes.c_void_p * n)(*[None if a is None else a.ctypes.data for a in arrs])
            keep.append(t)
            tables[k] = ctypes.cast(t, ctypes.c_void_p)
        keep.append(tables)
        return ctypes.cast(tables, ctypes.c_void_p)

    def _cached_tables(self, key, n, fields):
        """Pointer tables of `fields`, rebuilt only when the arrays are not
        the very objects of the previous call (a batch cycled in place passes
        the same arrays every step)."""
        arrs = [f.get(name) for f in fields for name in FIELD_NAMES]
        cache = self.__dict__.setdefault("_tcache", {})
        hit = cache.get(key)
        if hit is not None and len(hit[0]) == len(arrs) and all(x is y for x, y in zip(hit[0], arrs)):
            return hit[1]
        for a in arrs:
            if a is not None and (a.dtype != np.float64 or not a.flags.c_contiguous):
                raise ValueError("cycle needs C-contiguous float64 arrays")
        keep = []
        tables = self._tables(n, fields, keep)
        cache[key] = (arrs, tables, keep)
        return tables

    def _many(self, fn, slots, fields):
        n = len(slots)
        keep = []
        tables = self._tables(n, fields, keep)
        sl = np.ascontiguousarray(slots, dtype=np.int32)
        check(fn(self._h, n, _p(sl), tables))

    def cycle(self, slots, fields_in, nsweeps, fields_out=None, graph=True):
        """One pipelined batch (su2gpu_pool_cycle): upload every active
        chain's fields, `nsweeps` sweeps, measurement, download into
        fields_out (default: in place into fields_in).  Returns the
        measurement sums, one row per slot."""
        fields_out = fields_in if fields_out is None else fields_out
        n = len(slots)
        tin = self._cached_tables("in", n, fields_in)
        tout = self._cached_tables("out", n, fields_out)
        sums = np.zeros((n, abi.NMEAS))
        sl = np.ascontiguousarray(slots, dtype=np.int32)
        check(lib().su2gpu_pool_cycle(self._h, n, _p(sl), tin, nsweeps, 1 if graph else 0, _p(sums), tout))
        return sums

    def upload_many(self, slots, fields):
        """Upload the chains `slots` in one call; fields[j] is a dict of
        C-contiguous float64 arrays (as `upload`) for slots[j]."""
        for f in fields:
            for a in f.values():
                if a is not None and (a.dtype != np.float64 or not a.flags.c_contiguous):
                    raise ValueError("upload_many needs C-contiguous float64 arrays")
        self._many(lib().su2gpu_pool_upload_many, slots, fields)

    def download_many(self, slots, fields):
        """Download the chains `slots` in one call into the arrays of
        fields[j] (dicts as `download(out=...)` takes)."""
        for s, f in zip(slots, fields):
            shapes = _shapes(self._params[s])
            for n, a in f.items():
                if a is not None and (a.shape != shapes[n] or a.dtype != np.float64 or not a.flags.c_contiguous):
                    raise ValueError(f"{n}: need a C-contiguous float64 array of shape {shapes[n]}")
        self._many(lib().su2gpu_pool_download_many, slots, fields)

    def set_sweep(self, slot, sweep):
        check(lib().su2gpu_pool_set_sweep(self._h, slot, sweep))

    def run(self, nsweeps, graph=True):
        check(lib().su2gpu_pool_run(self._h, nsweeps, 1 if graph else 0))

    def measure(self):
        """{slot: measure() sums} of every active chain."""
        slots = self.active()
        out = np.zeros((max(len(slots), 1), abi.NMEAS))
        n = ctypes.c_int32()
        check(lib().su2gpu_pool_measure(self._h, _p(out), out.shape[0], ctypes.byref(n)))
        return {int(s): out[k].copy() for k, s in enumerate(slots)}

    def enqueue(self, nsweeps, graph=True):
        check(lib().su2gpu_pool_enqueue(self._h, nsweeps, 1 if graph else 0))

    @property
    def persistent(self):
        """Whether the sweeps run as one launch of the persistent work-list
        kernel rather than one launch per pass, for the current chains."""
        on = ctypes.c_int32()
        check(lib().su2gpu_pool_get_persistent(self._h, ctypes.byref(on)))
        return bool(on.value)

    @persistent.setter
    def persistent(self, on):
        """True / False force the mode; None: automatic (the default,
        persistent from 8 chains on)."""
        check(lib().su2gpu_pool_set_persistent(self._h, -1 if on is None else (1 if on else 0)))

    @property
    def persist_tiles(self):
        """Tiles of 128 sites per work item of the persistent sweep."""
        n = ctypes.c_int32()
        check(lib().su2gpu_pool_get_persist_tiles(self._h, ctypes.byref(n)))
        return n.value

    @property
    def persist_shape(self):
        """(shape, threads, resident blocks per SM) of the persistent sweep."""
        a, b, c = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        check(lib().su2gpu_pool_get_persist_shape(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    @persist_shape.setter
    def persist_shape(self, shape):
        check(lib().su2gpu_pool_set_persist_shape(self._h, int(shape)))

    @property
    def sweep_groups(self):
        """(groups, streams) of the grouped sweep mode in effect ((0, 1): off)."""
        g, n = ctypes.c_int32(), ctypes.c_int32()
        check(lib().su2gpu_pool_get_sweep_groups(self._h, ctypes.byref(g), ctypes.byref(n)))
        return g.value, n.value

    @sweep_groups.setter
    def sweep_groups(self, gs):
        """(groups, streams); None or groups <= 1: off."""
        g, n = (0, 1) if gs is None else gs
        check(lib().su2gpu_pool_set_sweep_groups(self._h, int(g), int(n)))

    def check_wait_timeout(self, spin_limit=2000):
        """Run the persistent kernel on a work list whose dependencies never
        finish; returns the kernel's error flags (4: a wait gave up)."""
        flags = ctypes.c_int32()
        check(lib().su2gpu_pool_check_wait_timeout(self._h, spin_limit, ctypes.byref(flags)))
        return flags.value

    def muca_set(self, slot, weight_struct):
        """Give chain `slot` a multicanonical weight (su2gpu_weight)."""
        check(lib().su2gpu_pool_muca_set(self._h, slot, ctypes.byref(weight_struct)))

    def muca_get(self, slot, weight_struct):
        check(lib().su2gpu_pool_muca_get(self._h, slot, ctypes.byref(weight_struct)))

    def calc_orderparam(self, slot, parity):
        v = ctypes.c_double(0)
        check(lib().su2gpu_pool_calc_orderparam(self._h, slot, parity, ctypes.byref(v)))
        return v.value

    def raise_error(self, flags):
        """Test hook: set error flags in the pool's device error word."""
        check(lib().su2gpu_pool_raise_error(self._h, flags))

    def enqueue_measure(self, device_ptr, max_chains):
        """Measurement of every active chain into a device buffer of
        max_chains * NMEAS doubles (asynchronous); returns the chain count."""
        n = ctypes.c_int32()
        check(lib().su2gpu_pool_enqueue_measure(self._h, ctypes.c_void_p(device_ptr), max_chains, ctypes.byref(n)))
        return n.value

    def set_stream(self, stream_ptr):
        check(lib().su2gpu_pool_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)))

    def launches_per_sweep(self):
        n = ctypes.c_int32()
        check(lib().su2gpu_pool_launches_per_sweep(self._h, ctypes.byref(n)))
        return n.value

    def profile_sweep(self, max_passes=512):
        kinds = np.zeros(max_passes, dtype=np.int32)
        ms = np.zeros(max_passes, dtype=np.float32)
        n = ctypes.c_int32()
        check(lib().su2gpu_pool_profile_sweep(self._h, max_passes, _p(kinds), _p(ms), ctypes.byref(n)))
        return kinds[:n.value], ms[:n.value]

    def counters(self, slot):
        out = np.zeros(abi.NCOUNTERS, dtype=np.int64)
        check(lib().su2gpu_pool_counters(self._h, slot, _p(out)))
        return out

    def autotune(self):
        ch = np.zeros(5, dtype=np.int32)
        ms = np.zeros(5, dtype=np.float32)
        check(lib().su2gpu_pool_autotune(self._h, _p(ch), _p(ms)))
        return ch, ms

    def set_variants(self, choices):
        ch = np.ascontiguousarray(choices, dtype=np.int32)
        check(lib().su2gpu_pool_set_variants(self._h, _p(ch)))

    def extract(self, slot):
        """The chain copied into a `Lattice` of its own (same parameters,
        seed and chain id); the chain stays in the pool."""
        h = ctypes.c_void_p()
        check(lib().su2gpu_pool_extract(self._h, slot, ctypes.byref(h)))
        return Lattice(self._params[slot], _handle=h)

    def grad_flow(self, slot, t_max, dt, meas_interval=1):
        maxrows = int(np.ceil(t_max / dt)) // meas_interval + 3
        rows = np.zeros((maxrows, 1 + abi.NMEAS))
        n = ctypes.c_int32()
        check(lib().su2gpu_pool_grad_flow(self._h, slot, t_max, dt, meas_interval, _p(rows), maxrows,
                                          ctypes.byref(n)))
        return rows[:n.value]
