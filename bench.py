#!/usr/bin/env python3
"""Throughput of the su2higgs checkerboard update sweep on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference] [--workload NAME]

Default workload, batched384_adj_f32 -- the FP32 batched form: 384 independent
SU(2) + adjoint Higgs chains (side L uniform over {8,12,16,24,32,48}, beta
uniform in [6,12], m^2_adj scanning [-0.3,0.1], lambda_adj 0.005; 11.0 M sites
in all) resident in one device pool.  A step is 10 sweeps of every chain (6
link heatbath + 10 triplet half-sweeps each) as one graph-replayed launch of
the persistent work-list kernel, followed by the measurement of every chain;
the default 100 steps are the workload's 1000 sweeps per chain.
Single-lattice workloads (fund128_f32 ...): a step is one sweep of SU(2) +
fundamental Higgs plus its measurement.

value      site-updates/s = sites * sweeps / (sum of per-step CUDA-event
           times on the launching stream); the fields (660 MB for the
           ensemble, 128 MB+ for 128^3) exceed the 126 MB L2 and a 256 MiB
           write flushes L2 between steps, outside the events
e2e        the same metric through the host-buffer C ABI (FP64 AoS host
           arrays, page-locked): upload of every chain + sweeps + measure +
           download per step, wall clock; the batched workloads make one
           su2gpu_pool_cycle call per step (groups of chains pipelined over
           the copy engines and the update kernels)
fp64_plain the plain FP64 single-lattice sweep on the same lattices run one
           after another (the metric's comparison)
roofline   the dominant kernel: for a pool in the persistent mode the
           work-list kernel (CUDA events on its stream around launches of
           the step's sweeps), with the one-launch-per-pass profile beside
           it; otherwise the kernel kind with the largest share of profiled
           sweeps (CUDA events around every pass on the launching stream)
cpu_baseline  the oracle's C restatement of the sweep, one thread, on a
           bounded sample of the same lattices

--impl reference runs that CPU restatement on all host cores instead (one
independent lattice per core; the reference itself is serial C).
Under torchrun each rank runs an independent replica (weak scaling).
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "site-updates/s, FP32 batched vs FP64 plain (same GB300); p50/p99 chain latency"

WORKLOADS = {
    # name: (content, L, precision)
    "fund128_f32": ("fund", (128, 128, 128), 32),
    "fund128_f64": ("fund", (128, 128, 128), 64),
    "fund64_f32": ("fund", (64, 64, 64), 32),
    "fund64_f64": ("fund", (64, 64, 64), 64),
    "fund16_f64": ("fund", (16, 16, 16), 64),
    "fund160_f32": ("fund", (160, 160, 160), 32),
    # multicanonical SU(2) x U(1) + singlet, 96^3, beta_G 8, beta_U1 24: a
    # seeded piecewise-linear weight over phi^2 (256 bins on [0, 3]), one
    # global accept/reject per Higgs sweep; a gradient flow t = 0..4, step
    # 0.01, timed after the sweeps
    "muca96_su2u1s_f32": ("su2u1s", (96, 96, 96), 32),
}

BATCHED = {
    # name: (chains, sweeps per step)
    "batched384_adj_f32": (384, 10),
    "batched96_adj_f32": (96, 10),
}

# Compulsory device traffic per lattice site, in reals, for one launch of each
# pass kind (each array element a launch must touch counted once).
# Fundamental content: link heatbath reads the two other directions everywhere
# (8), the updated direction at the other parity (2; the heatbath draw does not
# depend on the old link), writes half of it (2) and reads the doublet
# everywhere (4) -> 16; a doublet pass reads the doublet everywhere (4), all
# links (12) and writes half the doublet (2) -> 18.  Adjoint content: the link
# update reads the updated direction everywhere (its Metropolis correction
# needs the old link): 8 + 4 + 2 + the triplet everywhere (3) -> 17; a triplet
# pass reads all links (12) and the triplet everywhere (3) and writes half of
# it (1.5) -> 16.5.
# SU(2) x U(1) + singlet content: the SU(2) link heatbath reads the two other
# directions (8), the updated one at the other parity (2), the doublet (4) and
# the U(1) angle of the updated direction at the updated sites (0.5), and
# writes half the direction (2) -> 16.5; a U(1) pass reads the angles of the
# two other directions (2), the updated one everywhere and writes half (1.5),
# the doublet (4) and the SU(2) link at the updated sites (2) -> 9.5; a
# doublet pass reads all links (12), all angles (3), the doublet everywhere
# (4), the singlet at the updated sites (0.5), writes half the doublet (2) and,
# multicanonical, its backup (2) -> 23.5; a singlet pass reads the singlet
# everywhere (1) and the doublet at the updated sites (2), writes half (0.5)
# -> 3.5.
REALS_PER_SITE = {"fund": {0: 16, 2: 18}, "adj": {0: 17, 3: 16.5}, "su2u1s": {0: 16.5, 1: 9.5, 2: 23.5, 4: 3.5}}
# Compulsory reals per site of the passes of one sweep (6 link half-passes,
# 10 scalar half-passes) and of one measurement reading every field once; a
# site-update counts the measurement at the workload's cadence (once per
# sweep for the single lattices, once per step of S sweeps in the batched
# form)
REALS_PER_SWEEP = {"fund": 6 * 16 + 10 * 18, "adj": 6 * 17 + 10 * 16.5,
                   "su2u1s": 6 * 16.5 + 6 * 9.5 + 10 * 23.5 + 10 * 3.5}
REALS_MEASURE = {"fund": 16, "adj": 15, "su2u1s": 20}
KIND_NAMES = {0: "link_heatbath", 1: "u1_metropolis", 2: "doublet_update", 3: "triplet_update",
              4: "singlet_update", 5: "reunitarize"}


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def replica_seed(base, rank):
    """Seed of a rank's replica: independent chains per rank (weak scaling)."""
    return base + 1000003 * rank


def max_over_ranks(ms, dist, device):
    """The slowest rank's time (every rank gets it); ms itself without ranks."""
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    if dist:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate(units_per_rank, world, ms):
    """Whole-job throughput: the units every rank processed over the slowest
    rank's time."""
    return world * units_per_rank / (ms * 1e-3)


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.file.flush()
        rows = []
        with open(self.file.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        smax = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def hot_fields(p, seed):
    from su2higgs_gb300 import abi
    rng = np.random.default_rng(seed)
    V = p.sites()
    link = rng.normal(size=(V, 3, 4))
    link /= np.linalg.norm(link, axis=2, keepdims=True)
    out = {"link": link}
    if p.nhiggs() > 0:
        out["d0"] = rng.normal(scale=0.1, size=(V, 4))
    if p.content & abi.TRIPLET:
        out["trip"] = rng.normal(scale=0.1, size=(V, 3))
    return out


def cpu_sample_sweeps(content, L, seed, nsweeps=1):
    """Time the oracle's C restatement (one thread): nsweeps sweeps + measure."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from native import Fields, Oracle
    from su2higgs_gb300 import abi
    p = abi.make_params(content, L=L)
    f = hot_fields(p, seed)
    o = Oracle(p)
    o.put(Fields(p, link=f["link"], d0=f.get("d0"), trip=f.get("trip")))
    o.set_rng(seed, 0)
    t0 = time.perf_counter()
    for s in range(nsweeps):
        o.set_rng(seed, s)
        o.update()
        o.measure()
    return p.sites() * nsweeps, time.perf_counter() - t0


def _cpu_worker(args):
    content, L, seed, nsweeps = args
    return cpu_sample_sweeps(content, L, seed, nsweeps)


def _cpu_chain_worker(args):
    """One sweep + measure of one ensemble chain with the oracle (FP64)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from native import Fields, Oracle
    from su2higgs_gb300 import abi, workloads
    content, L, beta, msq, seed, chain = args
    kw = dict(msq_triplet=msq, b4=0.005) if content == "adj" else dict(msq_phi=msq)
    p = abi.make_params(content, L=(L, L, L), precision=64, betasu2=beta, **kw)
    f = workloads.hot_fields(p, seed)
    o = Oracle(p)
    o.put(Fields(p, **f))
    o.set_rng(seed, 0, chain)
    t0 = time.perf_counter()
    o.update()
    o.measure()
    return p.sites(), time.perf_counter() - t0, os.getpid()


def batched_config(workload, specs):
    """The workload's description, the same on both arms (the GPU arm's
    launch details are reported beside it, under "step")."""
    from su2higgs_gb300 import workloads
    Ls = [int(p.L[0]) for p, _, _ in specs]
    return {"workload": workload, "content": "SU(2) + adjoint Higgs", "chains": len(specs),
            "sites_total": int(sum(p.sites() for p, _, _ in specs)),
            "sides": {str(L): Ls.count(L) for L in sorted(set(Ls))},
            "betasu2": list(workloads.ENSEMBLE_BETA), "msq_adj": list(workloads.ENSEMBLE_MSQ_ADJ),
            "lambda_adj": workloads.ENSEMBLE_LAMBDA_ADJ, "sweeps_per_chain": 1000,
            "recipe": "1 link heatbath (3 directions x 2 parities) + 4 triplet overrelax + 1 triplet Metropolis "
                      "(x 2 parities) per sweep; every chain measured once per 10 sweeps",
            "start": "seeded hot start (Haar links, triplet N(0, 0.1))"}


def _cpu_ensemble_worker(args):
    """One sweep (+ the measurement, when `measure`) of one ensemble chain
    with the oracle (FP64), from its seeded start."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from native import Fields, Oracle
    from su2higgs_gb300 import abi, workloads
    L, beta, msq, b4, seed, chain, measure = args
    p = abi.make_params("adj", L=(L, L, L), precision=64, betasu2=beta, msq_triplet=msq, b4=b4)
    f = workloads.hot_fields(p, seed)
    o = Oracle(p)
    o.put(Fields(p, **f))
    o.set_rng(seed, 0, chain)
    t0 = time.perf_counter()
    o.update()
    if measure:
        o.measure()
    return p.sites(), time.perf_counter() - t0, os.getpid()


def run_reference_batched(args):
    """The oracle's FP64 restatement of the reference's serial sweep on all
    host cores: each step sweeps 4 x cores chains of the ensemble (cycling
    through it), one process per core, largest first so that the cores stay
    balanced as they would over a long run; a step lasts as long as the
    busiest core's sweeps (set-up excluded, as on the GPU)."""
    from su2higgs_gb300 import serve, workloads
    import multiprocessing as mp
    if args.workload == "served":
        # requests with L <= 32 only, so that a step stays well under a
        # second: the CPU sweep's cost per site does not depend on L
        stream = serve.make_stream(args.serve_rate, args.serve_window, seed=20261203)
        jobs = [(r.content, r.L, r.betasu2, r.msq, r.seed, r.rid) for r in stream if r.L <= 32]
        nchains, what = len(jobs), "requests (L <= 32) of the served stream"
    else:
        return run_reference_ensemble(args)
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    done, wall, nxt = 0, 0.0, 0
    per_step = 4 * cores
    with ctx.Pool(cores) as pool:
        for s in range(args.warmup + args.steps):
            batch = sorted((jobs[(nxt + k) % len(jobs)] for k in range(per_step)), key=lambda j: -j[1])
            nxt += per_step
            res = pool.map(_cpu_chain_worker, batch, chunksize=1)
            if s < args.warmup:
                continue
            per_pid = {}
            for n, t, pid in res:
                per_pid[pid] = per_pid.get(pid, 0.0) + t
            done += sum(r[0] for r in res)
            wall += max(per_pid.values())
    value = done / wall
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "site-updates/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "chains": nchains,
                   "sample": f"{per_step} {what} per step, one sweep + measure each"},
        "cpu_baseline": {"value": value, "unit": "site-updates/s", "cores": cores, "kind": "port",
                         "sample": f"{per_step} {what} per step (one process per core, cycling through "
                                   f"{nchains} of them), 1 sweep + measure each; oracle C restatement of the "
                                   "reference's serial sweep"},
        "e2e": {"value": value, "unit": "site-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_reference_ensemble(args):
    """The oracle's FP64 restatement of the reference's serial sweep on all
    host cores over the whole ensemble: each step sweeps every one of its
    chains once (one process per core, largest chains first, so that the
    cores stay balanced), measuring each chain once per 10 steps as the GPU
    arm measures once per 10 sweeps; a step lasts as long as the busiest
    core's sweeps (lattice set-up excluded, as on the GPU)."""
    from su2higgs_gb300 import workloads
    import multiprocessing as mp
    nchains, S = BATCHED[args.workload]
    specs = workloads.batched_ensemble(nchains)
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    done, wall = 0, 0.0
    with ctx.Pool(cores) as pool:
        for s in range(args.warmup + args.steps):
            jobs = sorted(((int(p.L[0]), float(p.betasu2), float(p.msq_triplet), float(p.b4), seed, chain,
                            s % S == S - 1) for p, seed, chain in specs), key=lambda j: -j[0])
            res = pool.map(_cpu_ensemble_worker, jobs, chunksize=1)
            if s < args.warmup:
                continue
            per_pid = {}
            for n, t, pid in res:
                per_pid[pid] = per_pid.get(pid, 0.0) + t
            done += sum(r[0] for r in res)
            wall += max(per_pid.values())
    value = done / wall
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "site-updates/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": batched_config(args.workload, specs),
        "step": {"sweeps_per_step": 1, "what": f"one sweep of all {nchains} chains, every 10th step with the "
                                              "measurement of every chain"},
        "cpu_baseline": {"value": value, "unit": "site-updates/s", "cores": cores, "kind": "port",
                         "sample": f"every step: one sweep of each of the {nchains} chains of the ensemble "
                                   f"(one process per core, {cores} processes), measured once per {S} steps; "
                                   "oracle C restatement of the reference's serial sweep in FP64"},
        "e2e": {"value": value, "unit": "site-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return
    if args.workload in BATCHED or args.workload == "served":
        return run_reference_batched(args)
    if args.workload == "batched96_su2u1s_muca_f32":
        # the chains' content and largest side; the CPU sample sweeps without
        # the multicanonical checks (a small share of the reference's time)
        content, L, prec = "su2u1s", (48, 48, 48), 32
    else:
        content, L, prec = WORKLOADS[args.workload]
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    # each step: every core sweeps its own lattice once; the lattice side is
    # chosen so that warm-up + steps stay within about two minutes
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        # calibrate the per-site cost on a 16^3 lattice
        n, t = pool.apply(_cpu_worker, (("fund", (16, 16, 16), 1, 1),))
        per_site = t / n
        budget = 120.0 / max(args.steps + args.warmup, 1)
        side = 16
        for cand in (128, 96, 64, 48, 32, 24, 16):
            if cand ** 3 * per_site <= budget and cand <= L[0]:
                side = cand
                break
        Ls = (side, side, side)
        for w in range(args.warmup):
            pool.map(_cpu_worker, [(content, Ls, 1000 + w * cores + k, 1) for k in range(cores)])
        done = 0
        wall = 0.0
        for s in range(args.steps):
            res = pool.map(_cpu_worker, [(content, Ls, 5000 + s * cores + k, 1) for k in range(cores)])
            done += sum(r[0] for r in res)
            # the workers sweep in parallel: a step lasts as long as the slowest
            # sweep (lattice set-up excluded, as the GPU arm's is)
            wall += max(r[1] for r in res)
    value = done / wall
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "site-updates/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "content": content, "lattice": list(L), "sample_lattice": list(Ls),
                   "recipe": "1 link heatbath + 4 doublet overrelax + 1 doublet Metropolis, measure each sweep"},
        "cpu_baseline": {"value": value, "unit": "site-updates/s", "cores": cores, "kind": "port",
                         "sample": f"{cores} independent {side}^3 lattices (one per core), 1 sweep + measure each per step; "
                                   "oracle C restatement of the reference's serial sweep"},
        "e2e": {"value": value, "unit": "site-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import torch
    from su2higgs_gb300 import abi, gpu

    rank, world, local = env_rank()
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    from su2higgs_gb300 import workloads
    content, L, prec = WORKLOADS[args.workload]
    muca = args.workload.startswith("muca")
    p = workloads.muca_params(prec) if muca else abi.make_params(content, L=L, precision=prec)
    V = p.sites()
    seed = replica_seed(20261203, rank)
    f = workloads.hot_fields(p, seed, phi_sigma=0.5, sing_sigma=0.3) if muca else hot_fields(p, seed)
    lat = gpu.Lattice(p, seed=seed, chain=rank)
    lat.upload(**f)
    weight = None
    if muca:
        weight = workloads.muca_weight(seed)
        lat.muca_set(weight.struct)
        lat.calc_orderparam(0)
        lat.calc_orderparam(1)
    if args.variants:
        variants = np.array([int(x) for x in args.variants.split(",")], dtype=np.int32)
        lat.set_variants(variants)
    else:
        variants, _ = lat.autotune()
    stream = torch.cuda.Stream(device=dev)
    lat.set_stream(stream.cuda_stream)
    K, W = args.steps, args.warmup
    sums = torch.zeros((K + W, abi.NMEAS), dtype=torch.float64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    launches_sweep = lat.launches_per_sweep()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    with torch.cuda.stream(stream):
        for w in range(W):
            lat.enqueue_sweeps(w, 1, graph=True)
            lat.enqueue_measure(sums[w].data_ptr())
            flush.zero_()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        clocks = ClockSampler(local)
        clocks.start()
        t_wall0 = time.perf_counter()
        for k in range(K):
            starts[k].record(stream)
            lat.enqueue_sweeps(W + k, 1, graph=True)
            lat.enqueue_measure(sums[W + k].data_ptr())
            ends[k].record(stream)
            flush.zero_()
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall0
        clk = clocks.stop()
    if dist:
        dist.barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    dev_ms = max_over_ranks(float(np.sum(step_ms)), dist, dev)
    value = aggregate(V * K, world, dev_ms)
    m_last = sums[W + K - 1].cpu().numpy()
    assert np.all(np.isfinite(m_last)), "non-finite measurement"

    # roofline: a profiled pass over a few of the same steps
    lat.set_stream(None)
    kinds_all, ms_all = [], []
    for k in range(min(K, 10)):
        kinds, ms = lat.profile_sweep(W + K + k)
        kinds_all.append(kinds)
        ms_all.append(ms)
    kinds = np.concatenate(kinds_all)
    ms = np.concatenate(ms_all)
    shares = {}
    for kd in np.unique(kinds):
        shares[int(kd)] = float(ms[kinds == kd].sum())
    top = max(shares, key=shares.get)
    nlaunch = int(np.sum(kinds == top))
    avg_ms = shares[top] / nlaunch
    rsize = 4 if prec == 32 else 8
    alg_bytes = REALS_PER_SITE[content].get(top, 18) * rsize * V
    achieved = alg_bytes / (avg_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = None
    tr_path = os.path.join(ROOT, "profiles", f"traffic_{args.workload}.json")
    if os.path.exists(tr_path):
        with open(tr_path) as fh:
            tr = json.load(fh).get(KIND_NAMES[top])
        traffic = tr
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": KIND_NAMES[top], "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": alg_bytes, "avg_launch_ms": avg_ms,
                "time_share": shares[top] / sum(shares.values()),
                "shares": {KIND_NAMES[k]: v / sum(shares.values()) for k, v in shares.items()}}

    # end to end through the host-buffer C ABI call (FP64 AoS host arrays)
    e2e = None
    if rank == 0 and not args.no_e2e:
        host = {k: np.ascontiguousarray(v) for k, v in f.items()}
        for a in host.values():
            gpu.host_register(a)
        lat2 = gpu.Lattice(p, seed=seed)
        n_e2e = max(3, min(K, 20))
        h2d = sum(a.nbytes for a in host.values())
        lat2.update_lattice_host(0, host)
        lat2.measure()
        t0 = time.perf_counter()
        for k in range(n_e2e):
            lat2.update_lattice_host(1 + k, host)
            lat2.measure()
        te = time.perf_counter() - t0
        for a in host.values():
            gpu.host_unregister(a)
        e2e = {"value": V * n_e2e / te, "unit": "site-updates/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": h2d + abi.NMEAS * 8, "steps": n_e2e}
        lat2.close()

    # multicanonical statistics of the timed sweeps, and the gradient flow
    muca_info = flow = None
    if muca:
        cnt = lat.counters()
        muca_info = {"bins": workloads.MUCA_BINS, "range": list(workloads.MUCA_RANGE), "orderparam": "phi^2",
                     "checks_per_higgs_sweep": 1, "mode": "read-only weight",
                     "checks": int(cnt[abi.C_TOTAL_MUCA]), "accepted": int(cnt[abi.C_ACC_MUCA]),
                     "phi2_last": float(lat.calc_orderparam(0))}
        if rank == 0:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rows = lat.grad_flow(4.0, 0.01, 10)
            tf = time.perf_counter() - t0
            flow = {"t_max": 4.0, "dt": 0.01, "steps": 400, "measurements": int(len(rows)), "ms": 1e3 * tf,
                    "site_steps_per_s": V * 400 / tf}

    # the plain FP64 sweep on the same lattice (the metric's comparison)
    fp64 = None
    if rank == 0 and prec == 32 and not args.no_fp64:
        p64 = workloads.muca_params(64) if muca else abi.make_params(content, L=L, precision=64)
        lat64 = gpu.Lattice(p64, seed=seed)
        lat64.upload(**f)
        if muca:
            lat64.muca_set(weight.struct)
            lat64.calc_orderparam(0)
            lat64.calc_orderparam(1)
        lat64.autotune()
        lat64.set_stream(stream.cuda_stream)
        n64 = max(3, min(K // 4, 25))
        with torch.cuda.stream(stream):
            for w in range(3):
                lat64.enqueue_sweeps(w, 1, graph=True)
                lat64.enqueue_measure(sums[0].data_ptr())
                flush.zero_()
            torch.cuda.synchronize()
            tot = 0.0
            for k in range(n64):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                lat64.enqueue_sweeps(3 + k, 1, graph=True)
                lat64.enqueue_measure(sums[0].data_ptr())
                b.record(stream)
                flush.zero_()
                torch.cuda.synchronize()
                tot += a.elapsed_time(b)
        v64 = V * n64 / (tot * 1e-3)
        fp64 = {"value": v64, "unit": "site-updates/s", "steps": n64, "fp32_over_fp64": value / world / v64}
        lat64.close()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        n, tcpu = cpu_sample_sweeps(content, L, seed, 1)
        cpu = {"value": n / tcpu, "unit": "site-updates/s", "cores": 1, "kind": "port",
               "sample": f"1 sweep + measure of the same {L[0]}^3 lattice, oracle C restatement, 1 thread ({tcpu:.1f} s)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "site-updates/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": dev_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if prec == 32 else "f64", "data": "synthetic",
            "config": {"workload": args.workload, "content": content, "lattice": list(L),
                       "precision": f"FP{prec} fields, FP64 reductions" if prec == 32 else "FP64",
                       "recipe": ("1 SU(2) link heatbath + 1 U(1) Metropolis + 4 doublet and singlet overrelax + "
                                  "1 Metropolis, a global multicanonical check after each doublet half-sweep, "
                                  "measure each sweep") if muca else
                                 "1 link heatbath + 4 doublet overrelax + 1 doublet Metropolis, measure each sweep",
                       "couplings": {"betasu2": p.betasu2, "betau1": p.betau1, "msq": p.msq_phi,
                                     "lambda": p.lambda_phi} if muca else
                                    {"betasu2": p.betasu2, "msq": p.msq_phi, "lambda": p.lambda_phi},
                       "reunitarize_interval": p.reunitarize_interval if prec == 32 else None,
                       "l2": "flushed between steps (256 MiB write outside the step events)",
                       "parallelism": f"replicas x{world}", "graph": True,
                       "launch_variants": [int(v) for v in variants]},
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "fp64_plain": fp64,
            "sweep_roofline": sweep_roofline(value / world, content, prec),
            "multicanonical": muca_info, "gradient_flow": flow,
            # per step: the sweep's kernels, the sweep-counter set/increment, measure + reduction
            "gpu_launches": int(K * (launches_sweep + 4)),
            "clocks": clk, "wall_s_timed_region": t_wall,
            "step_ms_p50": float(np.percentile(step_ms, 50)), "step_ms_p99": float(np.percentile(step_ms, 99)),
        }
        print(json.dumps(line), flush=True)
    lat.close()
    if dist:
        dist.destroy_process_group()


def sweep_roofline(site_updates_per_s, content, prec, sweeps_per_measure=1):
    """The whole sweep against HBM: site-updates/s x compulsory bytes per
    site-update (the sweep's passes + the measurement at its cadence of one
    per `sweeps_per_measure` sweeps) over the measured copy bandwidth (one
    GPU)."""
    rsize = 4 if prec == 32 else 8
    b = (REALS_PER_SWEEP[content] + REALS_MEASURE[content] / sweeps_per_measure) * rsize
    peak, kind = measured_peaks()
    achieved = site_updates_per_s * b / 1e9
    return {"bytes_per_site_update": b, "sweeps_per_measurement": sweeps_per_measure, "achieved": achieved,
            "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": kind}


def roofline_of(kinds, ms, content, prec, sites, workload):
    """The kernel kind with the largest time share, its algorithmic bytes per
    launch (REALS_PER_SITE x sites) over its mean launch time."""
    shares = {}
    for kd in np.unique(kinds):
        shares[int(kd)] = float(ms[kinds == kd].sum())
    top = max(shares, key=shares.get)
    nlaunch = int(np.sum(kinds == top))
    avg_ms = shares[top] / nlaunch
    rsize = 4 if prec == 32 else 8
    alg_bytes = REALS_PER_SITE[content].get(top, 18) * rsize * sites
    achieved = alg_bytes / (avg_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = None
    tr_path = os.path.join(ROOT, "profiles", f"traffic_{workload}.json")
    if os.path.exists(tr_path):
        with open(tr_path) as fh:
            traffic = json.load(fh).get(KIND_NAMES[top])
    tot = sum(shares.values())
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "kernel": KIND_NAMES[top], "peak_source": peak_kind,
            "algorithmic_bytes_per_launch": alg_bytes, "avg_launch_ms": avg_ms, "launches_profiled": nlaunch,
            "time_share": shares[top] / tot, "shares": {KIND_NAMES[k]: v / tot for k, v in shares.items()}}


def persistent_roofline(kinds, launch_ms, S, content, prec, sites, workload, step_ms, groups=None):
    """The persistent sweep kernel (one launch of S sweeps): algorithmic
    bytes of the S sweeps (every pass: REALS_PER_SITE of its kind x sites;
    the passes of one sweep counted from a profiled per-pass sweep) over the
    median launch time.  groups = (G, NS): the grouped sweep instead, whose
    per-pass kernels of G groups overlap on NS streams -- the same bytes
    over the time of the S sweeps of all groups (fork to join)."""
    rsize = 4 if prec == 32 else 8
    kinds = np.asarray(kinds)
    nsw = max(1, int(np.sum(kinds == 0)) // 6)  # profiled sweeps (6 link passes each)
    per_sweep = sum(REALS_PER_SITE[content].get(int(k), 18) for k in kinds) / nsw * rsize * sites
    alg_bytes = per_sweep * S
    avg_ms = float(np.median(launch_ms))
    achieved = alg_bytes / (avg_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = None
    tr_path = os.path.join(ROOT, "profiles", f"traffic_{workload}.json")
    if os.path.exists(tr_path):
        with open(tr_path) as fh:
            tj = json.load(fh)
        if groups:
            # one grouped sweep's launches captured by ncu (serialised), else
            # the DRAM bytes of one launch of each kind over all chains
            t = tj.get("pool_sweep_grouped_per_sweep")
            per = [tj.get(KIND_NAMES.get(int(k), "")) for k in kinds]
            if t is not None:
                traffic = t * S
            else:
                traffic = None if any(x is None for x in per) else sum(per) / nsw * S
        else:
            t = tj.get("pool_sweep_persistent_per_sweep")
            traffic = None if t is None else t * S
    kernel = ("pool_sweep_persistent (k_pool_persist)" if not groups else
              f"pool sweep, grouped: k_pool_link / k_pool_scalar of {groups[0]} groups on {groups[1]} streams")
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "kernel": kernel, "peak_source": peak_kind,
            "algorithmic_bytes_per_launch": alg_bytes, "sweeps_per_launch": S, "avg_launch_ms": avg_ms,
            "launches_profiled": len(launch_ms), "time_share": min(1.0, avg_ms / step_ms)}


def cpu_sample_chains(specs, budget_s=15.0):
    """The oracle's C restatement, one thread: one sweep + measure of chains
    of the ensemble, smallest side first, until about budget_s seconds."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from native import Fields, Oracle
    from su2higgs_gb300 import abi, workloads
    order = sorted(range(len(specs)), key=lambda k: specs[k][0].L[0])
    # one chain of every side, then more of the same mix while time is left
    by_side = {}
    for k in order:
        by_side.setdefault(specs[k][0].L[0], []).append(k)
    picks = []
    for rnd in range(max(len(v) for v in by_side.values())):
        for side in sorted(by_side):
            if rnd < len(by_side[side]):
                picks.append(by_side[side][rnd])
    sites, t, used = 0, 0.0, []
    for k in picks:
        p, seed, chain = specs[k]
        p64 = abi.make_params("adj", L=tuple(p.L[:3]), precision=64, betasu2=p.betasu2,
                              msq_triplet=p.msq_triplet, b4=p.b4)
        f = workloads.hot_fields(p64, seed)
        o = Oracle(p64)
        o.put(Fields(p64, link=f["link"], trip=f["trip"]))
        o.set_rng(seed, 0, chain)
        t0 = time.perf_counter()
        o.update()
        o.measure()
        t += time.perf_counter() - t0
        sites += p64.sites()
        used.append(p.L[0])
        if t > budget_s:
            break
    return sites, t, used


def run_gpu_batched(args):
    import torch
    from su2higgs_gb300 import abi, gpu, workloads

    rank, world, local = env_rank()
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    nchains, S = BATCHED[args.workload]
    if args.sweeps_per_step:
        S = args.sweeps_per_step
    specs = workloads.batched_ensemble(nchains, seed=replica_seed(20261203, rank))
    sites = sum(p.sites() for p, _, _ in specs)
    arena = sum(gpu.Pool.chain_bytes(p) for p, _, _ in specs)
    pool = gpu.Pool(specs[0][0], arena_bytes=arena, max_chains=nchains)
    host = []
    for p, seed, chain in specs:
        slot = pool.add(p, seed=seed, chain=chain)
        f = workloads.hot_fields(p, seed)
        pool.upload(slot, **f)
        host.append((slot, f))
    if args.variants:
        variants = np.array([int(x) for x in args.variants.split(",")], dtype=np.int32)
        pool.set_variants(variants)
    else:
        variants, _ = pool.autotune()
    stream = torch.cuda.Stream(device=dev)
    pool.set_stream(stream.cuda_stream)
    K, W = args.steps, args.warmup
    sums = torch.zeros((2, nchains, abi.NMEAS), dtype=torch.float64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    launches_sweep = pool.launches_per_sweep()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    with torch.cuda.stream(stream):
        for w in range(W):
            pool.enqueue(S, graph=True)
            pool.enqueue_measure(sums[0].data_ptr(), nchains)
            flush.zero_()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        clocks = ClockSampler(local)
        clocks.start()
        t_wall0 = time.perf_counter()
        for k in range(K):
            starts[k].record(stream)
            pool.enqueue(S, graph=True)
            pool.enqueue_measure(sums[1].data_ptr(), nchains)
            ends[k].record(stream)
            flush.zero_()
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall0
        clk = clocks.stop()
    if dist:
        dist.barrier()
    pool.run(0)  # surfaces any error recorded by the kernels
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    dev_ms = max_over_ranks(float(np.sum(step_ms)), dist, dev)
    value = aggregate(sites * S * K, world, dev_ms)
    m_last = sums[1].cpu().numpy()
    assert np.all(np.isfinite(m_last)), "non-finite measurement"

    persistent = pool.persistent
    groups = pool.sweep_groups
    # the sweep kernels alone: S sweeps per launch (persistent mode: one
    # launch of the work-list kernel; grouped: the groups' graphs on several
    # streams, forked from and joined back into the pool's), CUDA events on the pool's stream,
    # inputs (660 MB) larger than L2 and the L2 flushed between launches
    sweep_ms = []
    with torch.cuda.stream(stream):
        for k in range(6):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            pool.enqueue(S, graph=True)
            b.record(stream)
            flush.zero_()
            sweep_ms.append((a, b))
        torch.cuda.synchronize()
    sweep_ms = [a.elapsed_time(b) for a, b in sweep_ms][1:]
    pool.set_stream(None)
    pool.run(0)
    kinds_all, ms_all = [], []
    for k in range(3):
        kd, ms = pool.profile_sweep()
        kinds_all.append(kd)
        ms_all.append(ms)
    kinds_all, ms_all = np.concatenate(kinds_all), np.concatenate(ms_all)
    per_pass = roofline_of(kinds_all, ms_all, "adj", 32, sites, args.workload)
    if persistent or groups[0] > 1:
        roofline = persistent_roofline(kinds_all, sweep_ms, S, "adj", 32, sites, args.workload,
                                       float(np.median(step_ms)), groups=None if persistent else groups)
        roofline["per_pass_mode"] = per_pass
    else:
        roofline = per_pass

    # end to end through the pool's host-buffer C ABI: every chain's FP64
    # fields uploaded from page-locked memory, S sweeps, measurement,
    # every chain downloaded, per step -- one su2gpu_pool_cycle call, which
    # pipelines groups of chains so that their host transfers run under the
    # sweeps of the others
    e2e = None
    if rank == 0 and not args.no_e2e:
        arrays = [a for _, f in host for a in f.values()]
        for a in arrays:
            gpu.host_register(a)
        h2d = sum(a.nbytes for a in arrays)
        n_e2e = max(3, min(K, 10))
        e2e_pool = gpu.Pool(specs[0][0], arena_bytes=arena, max_chains=nchains)
        e2e_pool.set_variants(variants)
        slots = [e2e_pool.add(p, seed=seed, chain=chain) for p, seed, chain in specs]

        fields = [f for _, f in host]

        def e2e_step():
            # in place: the step's results land in the same page-locked arrays
            e2e_pool.cycle(slots, fields, S)
        e2e_step()
        n_e2e = max(n_e2e, 20)
        tsteps = []
        # the interpreter's cyclic garbage collector is held off while the
        # steps are timed (a full collection over the harness's objects
        # took 100-200 ms inside one step); it runs before and after
        import gc
        gc.collect()
        gc.disable()
        try:
            for k in range(n_e2e):
                t0 = time.perf_counter()
                e2e_step()
                tsteps.append(time.perf_counter() - t0)
        finally:
            gc.enable()
        for a in arrays:
            gpu.host_unregister(a)
        # the host and its memory are shared with other jobs: a step now and
        # then takes longer for reasons outside this program, so the value is
        # taken from the median step time (the mean is reported beside it)
        t_med = float(np.median(tsteps))
        e2e = {"value": sites * S / t_med, "unit": "site-updates/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": h2d + nchains * abi.NMEAS * 8, "steps": n_e2e, "sweeps_per_step": S,
               "statistic": "median of the per-step wall times",
               "mean_value": sites * S * n_e2e / float(np.sum(tsteps)),
               "step_ms_p50": 1e3 * t_med, "step_ms_max": 1e3 * float(np.max(tsteps))}
        e2e_pool.close()

    # the plain FP64 sweep on the same lattices, one single-lattice context
    # after another (every 4th chain of the ensemble)
    fp64 = None
    if rank == 0 and not args.no_fp64:
        tot_sites, tot_ms = 0, 0.0
        n64 = 3
        with torch.cuda.stream(stream):
            for p, seed, chain in specs[::4]:
                p64 = abi.make_params("adj", L=tuple(p.L[:3]), precision=64, betasu2=p.betasu2,
                                      msq_triplet=p.msq_triplet, b4=p.b4)
                lat = gpu.Lattice(p64, seed=seed, chain=chain)
                lat.upload(**workloads.hot_fields(p64, seed))
                lat.set_stream(stream.cuda_stream)
                lat.enqueue_sweeps(0, 2, graph=True)
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                lat.enqueue_sweeps(2, n64, graph=True)
                lat.enqueue_measure(sums[0].data_ptr())
                b.record(stream)
                torch.cuda.synchronize()
                tot_ms += a.elapsed_time(b)
                tot_sites += p64.sites() * n64
                lat.close()
        v64 = tot_sites / (tot_ms * 1e-3)
        fp64 = {"value": v64, "unit": "site-updates/s", "chains": len(specs[::4]), "sweeps_each": n64,
                "fp32_batched_over_fp64_plain": value / world / v64,
                "what": "every 4th chain of the ensemble as an FP64 single-lattice context (graph replay), "
                        "one after another"}

    # the same ensemble in an FP64 pool, swept the same way (persistent
    # work list where the pool's rule picks it): separates the precision
    # gain from the batching gain
    fp64_batched = None
    if rank == 0 and not args.no_fp64:
        specs64 = workloads.batched_ensemble(nchains, seed=replica_seed(20261203, rank), precision=64)
        arena64 = sum(gpu.Pool.chain_bytes(p) for p, _, _ in specs64)
        pool64 = gpu.Pool(specs64[0][0], arena_bytes=arena64, max_chains=nchains)
        for p, seed, chain in specs64:
            slot = pool64.add(p, seed=seed, chain=chain)
            pool64.upload(slot, **workloads.hot_fields(p, seed))
        pool64.autotune()
        pool64.set_stream(stream.cuda_stream)
        ms64 = []
        with torch.cuda.stream(stream):
            for k in range(5):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                pool64.enqueue(S, graph=True)
                pool64.enqueue_measure(sums[0].data_ptr(), nchains)
                b.record(stream)
                flush.zero_()
                ms64.append((a, b))
            torch.cuda.synchronize()
        ms64 = [a.elapsed_time(b) for a, b in ms64][2:]
        pool64.set_stream(None)
        pool64.run(0)
        v64b = sites * S * len(ms64) / (sum(ms64) * 1e-3)
        fp64_batched = {"value": v64b, "unit": "site-updates/s", "steps": len(ms64), "sweeps_per_step": S,
                        "persistent": pool64.persistent, "fp32_over_fp64_batched": value / world / v64b,
                        "sweep_roofline": sweep_roofline(v64b, "adj", 64, sweeps_per_measure=S),
                        "what": "the same 384 chains in one FP64 pool, S sweeps + measurement per step "
                                "(CUDA events, L2 flushed between steps)"}
        pool64.close()

    # chain completion latency.  In the batched form every chain finishes
    # its 1000 sweeps at the same time, one ensemble step time x 100; the
    # served stream (continuous batching, requests of C5's mix arriving at
    # 1 per second, which one GPU sustains) gives the latency distribution
    latency = None
    if rank == 0 and not args.no_latency:
        from su2higgs_gb300 import serve
        t_chain = float(np.median(step_ms)) * 1e-3 * (1000 // S)
        stream_req = serve.make_stream(args.latency_rate, args.latency_window, seed=replica_seed(4242, rank))
        srv = serve.Server(gpu.Pool, gpu.Pool.chain_bytes, arena_bytes=int(8 << 30), max_chains=256,
                           quantum=args.serve_quantum)
        t0 = time.perf_counter()
        res = srv.serve(stream_req, deadline=args.latency_window + args.latency_drain)
        wall_l = time.perf_counter() - t0
        srv.close()
        lat_s = np.array([r.latency for r in res.values()]) if res else np.array([np.nan])
        latency = {"batched_chain_completion_s": t_chain,
                   "batched_what": f"every chain of the ensemble completes its 1000 sweeps together: "
                                   f"{1000 // S} steps x the median step time",
                   "served": {"arrival_rate_per_s": args.latency_rate, "arrival_window_s": args.latency_window,
                              "requests": len(stream_req), "completed": len(res), "unfinished": srv.unfinished,
                              "p50_latency_s": float(np.percentile(lat_s, 50)),
                              "p99_latency_s": float(np.percentile(lat_s, 99)),
                              "site_updates_per_s": srv.site_updates / wall_l,
                              "what": "served stream of the C5 request mix (L 16-128, fundamental / adjoint / "
                                      "SU(2)xU(1)+singlet, 500-5000 sweeps, 30% with a gradient flow), FP32"}}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        n, tcpu, used = cpu_sample_chains(specs)
        cpu = {"value": n / tcpu, "unit": "site-updates/s", "cores": 1, "kind": "port",
               "sample": f"1 sweep + measure of {len(used)} chains of the ensemble (sides {sorted(set(used))}), "
                         f"oracle C restatement in FP64, 1 thread ({tcpu:.1f} s)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "site-updates/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": dev_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": batched_config(args.workload, specs),
            "step": {"sweeps_per_step": S, "sweeps_per_chain_run": S * (K + W),
                     "precision": "FP32 fields, FP64 reductions",
                     "l2": "fields 660 MB > L2; 256 MiB write between steps outside the step events",
                     "parallelism": f"replicas x{world}", "graph": True,
                     "sweep_mode": "persistent work-list kernel, S sweeps per launch" if persistent
                     else (f"grouped: the chains in {groups[0]} groups of about equal sites, each group's "
                           f"S sweeps one launch per pass (a CUDA graph per group), the groups on {groups[1]} "
                           "streams in turn" if groups[0] > 1 else "one launch per pass"),
                     "sweep_groups": {"groups": groups[0], "streams": groups[1]} if groups[0] > 1 else None,
                     "persist_tiles_per_item": pool.persist_tiles if persistent else None,
                     "persist_shape": ({"shape": pool.persist_shape[0], "threads": pool.persist_shape[1],
                                        "blocks_per_sm": pool.persist_shape[2]} if persistent else None),
                     "launch_variants": [int(v) for v in variants]},
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "fp64_plain": fp64,
            "fp64_batched": fp64_batched, "latency": latency,
            "sweep_roofline": sweep_roofline(value / world, "adj", 32, sweeps_per_measure=S),
            # per step: the sweeps (persistent: one work-list kernel + the
            # sweep-counter increment; otherwise S graph replays of one
            # launch per pass) + measure + per-chain reduction
            "gpu_launches": int(K * ((launches_sweep if persistent else S * launches_sweep) + 2)),
            "clocks": clk, "wall_s_timed_region": t_wall,
            "step_ms_p50": float(np.percentile(step_ms, 50)), "step_ms_p99": float(np.percentile(step_ms, 99)),
        }
        print(json.dumps(line), flush=True)
    pool.close()
    if dist:
        dist.destroy_process_group()


def run_gpu_batched_muca(args):
    """Multicanonical chains in the batched form: 96 SU(2)xU(1) + doublet +
    singlet chains (sides 16..48, beta_G 8, beta_U1 24, FP32 fields), each
    with the multicanonical workload's read-only weight (256 bins of phi^2
    on [0, 3]) and a global check after every doublet half-sweep, in one
    pool; a step is 10 sweeps of every chain (the persistent sweep decides
    each chain's checks as its half-sweeps complete) + the measurement."""
    import torch
    from su2higgs_gb300 import abi, gpu, workloads
    rank, world, local = env_rank()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    rng = np.random.default_rng(replica_seed(777, rank))
    nchains, S = 96, 10
    specs = []
    for k in range(nchains):
        L = int(rng.choice((16, 24, 32, 48)))
        p = abi.make_params("su2u1s", L=(L, L, L), precision=32, betasu2=8.0, betau1=24.0)
        specs.append((p, int(rng.integers(1, 2 ** 62)), k))
    sites = sum(p.sites() for p, _, _ in specs)
    arena = sum(gpu.Pool.chain_bytes(p) for p, _, _ in specs)
    pool = gpu.Pool(specs[0][0], arena_bytes=arena, max_chains=nchains)
    weight = workloads.muca_weight(replica_seed(20261203, rank))
    slots = []
    for p, seed, chain in specs:
        s = pool.add(p, seed=seed, chain=chain)
        pool.upload(s, **workloads.hot_fields(p, seed, phi_sigma=0.5, sing_sigma=0.3))
        pool.muca_set(s, weight.struct)
        slots.append(s)
    variants, _ = pool.autotune()
    tuned = pool.persistent
    stream = torch.cuda.Stream(device=dev)
    K, W = args.steps, args.warmup
    sums = torch.zeros((nchains, abi.NMEAS), dtype=torch.float64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def timed(persistent):
        # W + K steps of S sweeps + the measurement in one sweep mode
        pool.persistent = persistent
        pool.set_stream(stream.cuda_stream)
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
        with torch.cuda.stream(stream):
            for w in range(W):
                pool.enqueue(S, graph=True)
                pool.enqueue_measure(sums.data_ptr(), nchains)
                flush.zero_()
            torch.cuda.synchronize()
            clocks = ClockSampler(local)
            clocks.start()
            for k in range(K):
                starts[k].record(stream)
                pool.enqueue(S, graph=True)
                pool.enqueue_measure(sums.data_ptr(), nchains)
                ends[k].record(stream)
                flush.zero_()
            torch.cuda.synchronize()
            clk = clocks.stop()
        pool.set_stream(None)
        pool.run(0)
        step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
        return sites * S * K / (float(np.sum(step_ms)) * 1e-3), step_ms, clk

    # the sweep mode the autotuner chose is the headline; the other is timed beside it
    other_value, _, _ = timed(not tuned)
    value, step_ms, clk = timed(tuned)
    launches_sweep = pool.launches_per_sweep()
    cnt = [pool.counters(s) for s in slots]
    pool.close()

    # the same chains without weights, for the cost of the checks
    pool = gpu.Pool(specs[0][0], arena_bytes=arena, max_chains=nchains)
    for p, seed, chain in specs:
        pool.upload(pool.add(p, seed=seed, chain=chain), **workloads.hot_fields(p, seed, phi_sigma=0.5, sing_sigma=0.3))
    pool.autotune()
    plain_tuned = pool.persistent
    plain_value, _, _ = timed(plain_tuned)
    pool.close()
    checks = int(sum(c[abi.C_TOTAL_MUCA] for c in cnt))
    accepted = int(sum(c[abi.C_ACC_MUCA] for c in cnt))
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "site-updates/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": float(np.mean(step_ms)), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "content": "SU(2)xU(1) + doublet + singlet", "chains": nchains,
                       "sites_total": sites, "sweeps_per_step": S, "betasu2": 8.0, "betau1": 24.0,
                       "weight": "read-only, 256 bins of phi^2 on [0, 3], one check per doublet half-sweep",
                       "persistent": tuned, "launch_variants": [int(v) for v in variants]},
            "multicanonical": {"checks": checks, "accepted": accepted},
            "other_sweep_mode": {"persistent": not tuned, "value": other_value},
            "without_weights": {"persistent": plain_tuned, "value": plain_value,
                                "what": "the same chains and fields in a pool without weights, autotuned"},
            "sweep_roofline": sweep_roofline(value / world, "su2u1s", 32, S),
            "gpu_launches": int(K * (launches_sweep if tuned else S * launches_sweep) + 2 * K),
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)


def run_gpu_served(args):
    """The served stream: Poisson arrivals of single-chain requests (side L
    in {16,32,64,96,128}, content fundamental / adjoint / SU(2)xU(1)+singlet,
    500-5000 sweeps, 30% with a gradient flow t = 0..4, dt = 0.01) played in
    real time through the continuous-batching server; arrivals stop after
    --serve-window seconds and the run ends --serve-drain seconds later."""
    from su2higgs_gb300 import abi, gpu, serve

    rank, world, local = env_rank()
    gpu.lib()
    rate, window, drain = args.serve_rate, args.serve_window, args.serve_drain
    stream = serve.make_stream(rate, window, seed=replica_seed(20261203, rank))
    arena = int(args.serve_arena_gb * (1 << 30))
    srv = serve.Server(gpu.Pool, gpu.Pool.chain_bytes, arena_bytes=arena, max_chains=1024,
                       quantum=args.serve_quantum)
    clocks = ClockSampler(local)
    clocks.start()
    t0 = time.perf_counter()
    res = srv.serve(stream, deadline=window + drain)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    srv.close()
    done = list(res.values())
    lat = np.array([r.latency for r in done]) if done else np.array([np.nan])
    offered = sum(r.sweeps * r.L ** 3 for r in stream) / window
    value = world * srv.site_updates / wall

    # the plain FP64 sweep run serially: one single-lattice FP64 context per
    # sampled request, a few sweeps each
    fp64 = None
    if rank == 0 and not args.no_fp64:
        tot_sites, tot_s = 0, 0.0
        sample = stream[:: max(1, len(stream) // 15)][:15]
        for r in sample:
            p64 = r.params(64)
            lat64 = gpu.Lattice(p64, seed=r.seed, chain=r.rid)
            n = 5
            lat64.run_sweeps(0, 1, graph=True)
            t1 = time.perf_counter()
            lat64.run_sweeps(1, n, graph=True)
            tot_s += time.perf_counter() - t1
            tot_sites += p64.sites() * n
            lat64.close()
        v64 = tot_sites / tot_s
        fp64 = {"value": v64, "unit": "site-updates/s", "requests_sampled": len(sample),
                "served_over_fp64_plain": value / world / v64,
                "what": "sampled requests as FP64 single-lattice contexts, 5 sweeps each, one after another"}
    d2h = sum(r.sums.nbytes + r.counters.nbytes + (0 if r.flow_rows is None else r.flow_rows.nbytes) for r in done)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "site-updates/s", "n_gpus": world, "steps": len(done),
            "warmup": 0, "ms_per_step": 1e3 * wall / max(len(done), 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "served", "arrival_rate_per_s": rate, "arrival_window_s": window,
                       "drain_s": drain, "requests": len(stream), "sides": list(serve.SIDES),
                       "contents": list(serve.CONTENTS), "sweeps": list(serve.SWEEPS),
                       "flow_fraction": serve.FLOW_FRACTION, "flow": serve.FLOW,
                       "arena_per_content_gb": args.serve_arena_gb, "quantum_sweeps": args.serve_quantum,
                       "precision": "FP32 fields, FP64 reductions", "start": "cold",
                       "parallelism": f"replicas x{world}"},
            "serving": {"completed": len(done), "unfinished": srv.unfinished,
                        "p50_latency_s": float(np.percentile(lat, 50)),
                        "p99_latency_s": float(np.percentile(lat, 99)),
                        "mean_queue_s": float(np.mean([r.admitted - r.arrival for r in done])) if done else None,
                        "offered_site_updates_per_s": offered, "achieved_over_offered": value / world / offered,
                        "completed_site_updates": int(sum(r.sweeps * r.sites for r in done))},
            "e2e": {"value": value, "unit": "site-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": d2h / max(len(done), 1),
                    "what": "wall clock of the whole served run: requests in, results (sums, counters, flow rows) "
                            "back to the host; chains start cold on the device"},
            "fp64_plain": fp64, "clocks": clk, "wall_s": wall,
        }
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="batched384_adj_f32",
                    choices=sorted(WORKLOADS) + sorted(BATCHED) + ["served", "batched96_su2u1s_muca_f32"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end host-buffer measurement")
    ap.add_argument("--no-latency", action="store_true", help="batched: skip the served latency leg")
    ap.add_argument("--latency-rate", type=float, default=1.0, help="batched latency leg: arrivals per second")
    ap.add_argument("--latency-window", type=float, default=20.0, help="batched latency leg: seconds of arrivals")
    ap.add_argument("--latency-drain", type=float, default=20.0,
                    help="batched latency leg: seconds after the last arrival")
    ap.add_argument("--sweeps-per-step", type=int, default=None,
                    help="batched: sweeps per step (default: the workload's 10; 1 for a profiler capture of one sweep)")
    ap.add_argument("--variants", default=None,
                    help="launch-shape variants of the 5 update kernel kinds, e.g. 0,0,0,0,0 (default: autotune)")
    ap.add_argument("--serve-rate", type=float, default=20.0, help="served: arrivals per second")
    ap.add_argument("--serve-window", type=float, default=30.0, help="served: seconds of arrivals")
    ap.add_argument("--serve-drain", type=float, default=30.0, help="served: seconds after the last arrival")
    ap.add_argument("--serve-arena-gb", type=float, default=24.0, help="served: device arena per content (GB)")
    ap.add_argument("--serve-quantum", type=int, default=50, help="served: sweeps per scheduling round")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload in BATCHED:
        run_gpu_batched(args)
    elif args.workload == "served":
        run_gpu_served(args)
    elif args.workload == "batched96_su2u1s_muca_f32":
        run_gpu_batched_muca(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
