"""Generate the golden fixtures in this directory from the reference itself.

Needs the reference harness built from the reference sources
(`make -C oracle/ref REF=<su2higgs checkout>`, outputs in oracle/_ref/).
Every fixture stores its inputs, so the tests never regenerate them:

  layout_<L>.npz         next/prev/coords/parity of layout() (layout.c:657-756)
  tables_sha256.npz      SHA-256 of those tables for the larger sides (up to 128^3)
  sites_<content>.npz    per-site staples, local actions, alpha_proj and
                         overrelaxation proposals (the value an accepted
                         overrelax_doublet / _higgs2 / _triplet / _singlet
                         writes, overrelax.c:54-417) on a hot lattice
  sweep_<case>.npz       fields + counters + measure() sums after 1 and 3 calls of
                         update_lattice() (update.c:270) with the Philox stream
  muca_<case>.npz        the same with multicanonical global accept/reject
  flow_<case>.npz        grad_flow() (gradflow.c:46) measurement rows
  mpi_layout.npz         the order in which N-rank runs write the sites of a
                         lattice file (write_field, checkpoint.c:226-269), from
                         the reference's MPI layout code (layout.c with -DMPI)
  correl_<case>.npz      measure_correlators() values (correlation.c:350-398) of
                         a hot lattice along the longest direction, and for
                         each blocking level (smear_fields + make_blocked_fields,
                         su2u1.c:857, blocking.c:296) the blocked links, triplet,
                         coordinates and correlator values

Run:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from native import Fields, Ref, hot_fields, layout_digest, ref_available, weight_from_state  # noqa: E402
from su2higgs_gb300 import abi  # noqa: E402

SEED = 20261203
LSMALL = (6, 4, 8)
CASES = {
    "pure": dict(content="pure"),
    "fund": dict(content="fund"),
    "adj": dict(content="adj"),
    "su2u1s": dict(content="su2u1s"),
    "fundadj": dict(content="fundadj"),
    "higgs2": dict(content="higgs2"),
    "fund_metro": dict(content="fund", algorithm_su2link=abi.METROPOLIS, algorithm_su2doublet=abi.METROPOLIS),
    "adj_metro": dict(content="adj", algorithm_su2triplet=abi.METROPOLIS),
    "su2u1s_metro": dict(content="su2u1s", algorithm_singlet=abi.METROPOLIS, algorithm_su2doublet=abi.METROPOLIS),
    "fund_upd2": dict(content="fund", update_links=2, scalar_sweeps=2, update_su2doublet=2),
}


def params(case, L=LSMALL):
    kw = dict(CASES[case])
    content = kw.pop("content")
    return abi.make_params(content, L=L, **kw)


def fields_dict(f, prefix):
    out = {}
    for name in ("link", "u1", "d0", "d1", "trip", "sing"):
        a = getattr(f, name)
        if a is not None:
            out[prefix + name] = a
    return out


def param_dict(p):
    return {"p_" + name: np.array(getattr(p, name) if name != "L" else list(p.L)) for name, _ in abi.Params._fields_
            if name != "reserved"}


# sides whose layout tables are stored as SHA-256 digests only
LAYOUT_HASHED = [(24, 24, 24), (48, 48, 48), (64, 64, 64), (96, 96, 96), (128, 128, 128), (32, 16, 24)]


def layout_hash_of(L):
    """The digest of one side's tables, each in a process of its own (the
    reference keeps its lattice in globals; large sides need an unlimited
    stack, as the reference's own runs do)."""
    import subprocess
    cmd = f"ulimit -s unlimited; {sys.executable} {os.path.abspath(__file__)} --layout-hash {L[0]} {L[1]} {L[2]}"
    out = subprocess.run(["bash", "-c", cmd], check=True, capture_output=True, text=True).stdout
    return out.strip().splitlines()[-1]


def gen_layout_hashes():
    Ls, digests = [], []
    for L in LAYOUT_HASHED:
        digests.append(layout_hash_of(L))
        Ls.append(L)
    np.savez_compressed(os.path.join(HERE, "tables_sha256.npz"), L=np.array(Ls, dtype=np.int32),
                        sha256=np.array(digests))


def gen_layout():
    for L in [(4, 4, 4), (6, 4, 8), (8, 8, 8), (2, 6, 4), (10, 2, 2), (12, 12, 12), (16, 16, 16)]:
        p = abi.make_params("pure", L=L)
        r = Ref(p)
        nx, pv, co, par = r.tables()
        name = "layout_" + "x".join(map(str, L)) + ".npz"
        np.savez_compressed(os.path.join(HERE, name), L=np.array(L), next=nx.astype(np.int32),
                            prev=pv.astype(np.int32), coords=co.astype(np.int32), parity=par)


def gen_sites(case):
    p = params(case)
    f = hot_fields(p, seed=SEED, phi_mean=0.5)
    r = Ref(p)
    r.put(f)
    V, D = r.V, p.dim
    import ctypes
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    out = dict(fields_dict(f, "in_"), **param_dict(p))
    st = np.zeros((V, D, 4))
    ws = np.zeros((V, D, 4))
    la = np.zeros((V, D))
    for i in range(V):
        for d in range(D):
            r.lib.ref_link_staple(i, d, P(st[i, d]))
            r.lib.ref_wilson_staple(i, d, P(ws[i, d]))
            la[i, d] = r.lib.ref_localact_su2link(i, d)
    out.update(link_staple=st, wilson_staple=ws, localact_su2link=la)
    out["action_local"] = np.array([r.lib.ref_action_local(i) for i in range(V)])
    out["local_su2wilson"] = np.array([r.lib.ref_local_su2wilson(i) for i in range(V)])
    if p.content & abi.U1:
        out["localact_u1link"] = np.array([[r.lib.ref_localact_u1link(i, d) for d in range(D)] for i in range(V)])
    if p.nhiggs():
        sd = np.zeros((V, 4))
        for i in range(V):
            r.lib.ref_staple_doublet(i, 0, P(sd[i]))
        out["staple_doublet"] = sd
        out["localact_doublet"] = np.array([r.lib.ref_localact_doublet(i, 0) for i in range(V)])
    if p.content & abi.TRIPLET:
        out["localact_triplet"] = np.array([r.lib.ref_localact_triplet(i) for i in range(V)])
        out["alpha_proj"] = np.array([[r.lib.ref_alpha_proj(i, a, b) for (a, b) in ((0, 1), (0, 2), (1, 2))]
                                      for i in range(V)])
        out["magcharge_cube"] = np.array([r.lib.ref_magcharge_cube(i) for i in range(V)])
    if p.content & abi.SINGLET:
        out["localact_singlet"] = np.array([r.lib.ref_localact_singlet(i) for i in range(V)])
    # overrelaxation proposals (every site, from the input fields)
    for key, kind, sub, n, present in (("or_doublet", 4, 0, 4, p.nhiggs() > 0),
                                       ("or_doublet1", 4, 1, 4, p.nhiggs() > 1),
                                       ("or_triplet", 6, 0, 3, bool(p.content & abi.TRIPLET)),
                                       ("or_singlet", 8, 0, 1, bool(p.content & abi.SINGLET))):
        if not present:
            continue
        a = np.zeros((V, n))
        for i in range(V):
            assert r.lib.ref_or_proposal(kind, i, sub, P(a[i])) == n
        out[key] = a if n > 1 else a[:, 0]
    out["measure"] = r.measure()
    np.savez_compressed(os.path.join(HERE, f"sites_{case}.npz"), **out)


def gen_sweep(case, seed=SEED + 1, first_sweep=5):
    p = params(case)
    f = hot_fields(p, seed=SEED, phi_mean=0.5)
    r = Ref(p)
    r.put(f)
    out = dict(fields_dict(f, "in_"), **param_dict(p))
    out["seed"] = np.array(seed, dtype=np.uint64)
    out["first_sweep"] = np.array(first_sweep)
    r.set_rng(seed, first_sweep)
    out["npasses"] = np.array(r.update())
    out.update(fields_dict(r.get(), "out1_"))
    out["counters1"] = r.counters()
    for s in (first_sweep + 1, first_sweep + 2):
        r.set_rng(seed, s)
        r.update()
    out.update(fields_dict(r.get(), "out3_"))
    out["counters3"] = r.counters()
    out["measure3"] = r.measure()
    np.savez_compressed(os.path.join(HERE, f"sweep_{case}.npz"), **out)


MUCA_CASES = {
    # name: (content, orderparam, mode, checks_per_sweep, nsweeps[, checks between weight updates])
    "su2u1s_phisq_ro": ("su2u1s", "phisq", 0, 1, 3),
    "su2u1s_phisq_fast": ("su2u1s", "phisq", 1, 1, 12),
    "fund_phisq_cps3": ("fund", "phisq", 1, 3, 4),
    "fund_phisq_cps5": ("fund", "phisq", 0, 5, 3),
    "adj_sigmasq_fast": ("adj", "Sigmasq", 1, 1, 12),
    "fundadj_p2ms2": ("fundadj", "phi2minusSigma2", 1, 2, 3),
    # two doublets, the order parameter on the second one (PHI2SQ)
    "higgs2_phi2sq_fast": ("higgs2", "phi2sq", 1, 2, 2),
    # the SLOW recursion (update_weight_slow): 60 checks a sweep, the weight
    # updated every 40 checks instead of the reference's 5000
    "fund_phisq_slow": ("fund", "phisq", 2, 5, 3, 40),
}


def gen_muca(name):
    content, op, mode, cps, nsweeps = MUCA_CASES[name][:5]
    interval = MUCA_CASES[name][5] if len(MUCA_CASES[name]) > 5 else None
    p = abi.make_params(content, L=LSMALL)
    f = hot_fields(p, seed=SEED + 7, phi_mean=0.5)
    # a weight around the starting order parameter, steep enough to reject often
    if op == "phisq":
        R0 = float(np.mean(0.5 * np.sum(f.d0 ** 2, axis=1)))
    elif op == "phi2sq":
        R0 = float(np.mean(0.5 * np.sum(f.d1 ** 2, axis=1)))
    elif op == "Sigmasq":
        R0 = float(np.mean(0.5 * np.sum(f.trip ** 2, axis=1)))
    else:
        R0 = float(np.mean(0.5 * np.sum(f.d0 ** 2, axis=1) - 0.5 * np.sum(f.trip ** 2, axis=1)))
    bins = 24
    lo, hi = R0 - 0.06, R0 + 0.06
    import tempfile
    wd = tempfile.mkdtemp(prefix="su2golden_")
    wpath = os.path.join(wd, "weight")
    rng = np.random.default_rng(SEED + 11)
    with open(wpath, "w") as fh:
        fh.write(f"{bins} 0.300000000000 0 {lo:f} {hi:f}\n")
        for k in range(bins + 1):
            pos = lo + k * (hi - lo) / bins
            W = 400.0 * (pos - lo) + 3.0 * rng.normal()
            fh.write(f"{pos:f} {W:f}\n")
    muca = dict(weightfile=wpath, muca_mode=mode, checks_per_sweep=cps, bins=bins, min=lo, max=hi,
                muca_delta=0.3, orderparam=op)
    r = Ref(p, workdir=wd, muca=muca)
    r.put(f)
    r.muca_init()
    if interval:
        r.muca_set_update_interval(interval)
    st0 = r.muca_state()
    out = dict(fields_dict(f, "in_"), **param_dict(p))
    for k, v in st0.items():
        out["w0_" + k] = np.asarray(v)
    seed = SEED + 3
    out["seed"] = np.array(seed, dtype=np.uint64)
    out["nsweeps"] = np.array(nsweeps)
    for s in range(nsweeps):
        r.set_rng(seed, 100 + s)
        r.update()
    out.update(fields_dict(r.get(), "out_"))
    out["counters"] = r.counters()
    st1 = r.muca_state()
    for k, v in st1.items():
        out["w1_" + k] = np.asarray(v)
    out["measure"] = r.measure()
    np.savez_compressed(os.path.join(HERE, f"muca_{name}.npz"), **out)


FLOW_CASES = {
    # name: (content, t_max, dt, meas_interval, identity_block)
    "fund": ("fund", 0.5, 0.05, 2, False),
    "adj": ("adj", 0.5, 0.05, 3, False),
    "su2u1s": ("su2u1s", 0.3, 0.07, 1, False),
    "fund_zeroforce": ("fund", 0.2, 0.05, 1, True),
}


def gen_flow(name):
    content, tmax, dt, mi, block = FLOW_CASES[name]
    p = abi.make_params(content, L=LSMALL)
    p.content |= abi.GRADFLOW
    f = hot_fields(p, seed=SEED + 21, phi_mean=0.5)
    if block:
        # identity links on a block of sites: links deep inside have exactly
        # zero force, which stops the reference's flow_gauge loop early
        # (gradflow.c:377-381)
        r0 = Ref(p)
        _, _, co, _ = r0.tables()
        inside = (co[:, 0] >= 1) & (co[:, 0] <= 4) & (co[:, 1] >= 0) & (co[:, 2] >= 2) & (co[:, 2] <= 6)
        f.link[inside] = np.array([1.0, 0, 0, 0])
    flow = dict(flow_t_max=tmax, flow_dt=dt, flow_meas_interval=mi)
    r = Ref(p, flow=flow)
    r.put(f)
    rows = r.grad_flow(tmax, dt)
    out = dict(fields_dict(f, "in_"), **param_dict(p))
    out["rows_raw"] = rows
    out["t_max"], out["dt"], out["meas_interval"] = np.array(tmax), np.array(dt), np.array(mi)
    # one Euler step of the fields themselves
    r.lib.ref_flow_step(dt)
    out.update(fields_dict(r.get(), "step_"))
    np.savez_compressed(os.path.join(HERE, f"flow_{name}.npz"), **out)


CORREL_CASES = {
    # name: (content, reference variant, L, blocking levels asked for)
    "adj_6x4x8": ("adj", "adjc", (6, 4, 8), 2),
    "adj_8x8x12": ("adj", "adjc", (8, 8, 12), 2),
    "adj_12x8x8": ("adj", "adjc", (12, 8, 8), 2),
    "fundadj_8x6x10": ("fundadj", "fundadjc", (8, 6, 10), 0),
    "fund_6x8x4": ("fund", "fundc", (6, 8, 4), 0),
}


def gen_correl(name):
    content, variant, L, levels = CORREL_CASES[name]
    p = abi.make_params(content, L=L)
    f = hot_fields(p, seed=SEED + 21, trip_sigma=0.5, phi_mean=0.4)
    r = Ref(p, variant=variant)
    r.put(f)
    ld = r.longest_dir()
    out = dict(fields_dict(f, "in_"), **param_dict(p))
    out["dir"] = np.array(ld)
    out["corr0"] = r.correlators(ld)
    n = r.block_setup(levels) if levels else 0
    out["levels"] = np.array(n)
    for k in range(n):
        b = r.blocked_level(k, ld)
        for key in ("corr", "link", "trip", "coords", "L"):
            out[f"b{k + 1}_{key}"] = b[key]
    np.savez_compressed(os.path.join(HERE, f"correl_{name}.npz"), **out)


MPI_LAYOUTS = [((6, 4, 8), n) for n in (2, 3, 4, 6, 8, 12, 16)] + [((8, 8, 8), 4), ((10, 6, 12), 15),
                                                                   ((16, 8, 12), 12)]


def gen_mpi_layout():
    import ctypes
    lib = ctypes.CDLL(os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle", "_ref", "libref_mpilayout.so"))
    lib.ref_mpi_rank_sites.restype = ctypes.c_long
    out = {}
    for L, n in MPI_LAYOUTS:
        V = int(np.prod(L))
        parts = []
        for r in range(n):
            co = np.zeros(V * 3, np.int64)
            ns = np.zeros(3, np.int32)
            k = lib.ref_mpi_rank_sites(3, (ctypes.c_int * 3)(*L), n, r, co.ctypes.data_as(ctypes.c_void_p),
                                       ns.ctypes.data_as(ctypes.c_void_p))
            parts.append(co[: k * 3].reshape(k, 3))
        co = np.concatenate(parts)
        name = "x".join(map(str, L)) + f"_{n}"
        # lexicographic index of every file position
        out["order_" + name] = co[:, 0] + L[0] * (co[:, 1] + L[1] * co[:, 2])
        out["nslices_" + name] = ns
    np.savez_compressed(os.path.join(HERE, "mpi_layout.npz"), **out)


def main(only=None):
    if only:
        for m in only:
            if m == "mpi_layout":
                gen_mpi_layout()
            elif m == "layout":
                gen_layout()
                gen_layout_hashes()
            elif m.startswith("sites_"):
                gen_sites(m[len("sites_"):])
            elif m in CORREL_CASES:
                gen_correl(m)
            else:
                gen_muca(m)
        return
    if not ref_available("fund"):
        sys.exit("reference harness not built: make -C oracle/ref REF=<su2higgs checkout>")
    gen_layout()
    gen_layout_hashes()
    for c in ("pure", "fund", "adj", "su2u1s", "fundadj", "higgs2"):
        gen_sites(c)
    for c in CASES:
        gen_sweep(c)
    for m in MUCA_CASES:
        gen_muca(m)
    for fl in FLOW_CASES:
        gen_flow(fl)
    for c in CORREL_CASES:
        gen_correl(c)
    gen_mpi_layout()
    total = sum(os.path.getsize(os.path.join(HERE, x)) for x in os.listdir(HERE) if x.endswith(".npz"))
    print(f"golden fixtures written, {total / 1024:.0f} KiB")


if __name__ == "__main__":
    if len(sys.argv) == 5 and sys.argv[1] == "--layout-hash":
        r = Ref(abi.make_params("pure", L=tuple(int(x) for x in sys.argv[2:5])))
        print(layout_digest(*r.tables()))
    else:
        main(sys.argv[1:])
