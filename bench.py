#!/usr/bin/env python3
"""Throughput of the su2higgs checkerboard update sweep on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference] [--workload NAME]

A step is one full sweep of the update recipe of the workload (link heatbath
for every direction and parity, 4 overrelaxation + 1 Metropolis passes of the
Higgs doublet) followed by one measurement of all volume sums, on a device-
resident lattice.  The default workload is the FP32 precision form at scale:
SU(2) + fundamental Higgs on 128^3, beta = 8, m^2 = -0.1, lambda = 0.002,
seeded hot start, links re-normalised every 10 sweeps, FP64 sums.

value      site-updates/s = V * K / (sum of per-step CUDA-event times); an L2
           flush (a 256 MiB write) runs between steps, outside the events
e2e        the same metric through the host-buffer C ABI call
           su2gpu_update_lattice_host (FP64 AoS host arrays, page-locked):
           upload + sweep + download + measure per step, wall clock
roofline   the kernel kind with the largest share of a profiled pass of the
           same steps (CUDA events around every pass on the launching stream)
cpu_baseline  the oracle's C restatement of the sweep, one thread, one sweep
           of the same lattice on the host cores

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
}

# Compulsory device traffic per lattice site, in reals, for one launch of each
# pass kind of the fundamental content (each array element a launch must touch
# counted once): link heatbath reads the two other directions everywhere (8),
# the updated direction everywhere and writes half of it (4 + 2), the doublet
# everywhere (4) -> 18; a doublet pass reads the doublet everywhere (4), all
# links (12) and writes half the doublet (2) -> 18; the measurement reads every
# field once (16).
REALS_PER_SITE = {0: 18, 2: 18}
REALS_MEASURE = 16
KIND_NAMES = {0: "link_heatbath", 1: "u1_metropolis", 2: "doublet_update", 3: "triplet_update",
              4: "singlet_update", 5: "reunitarize"}


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


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


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return
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
    content, L, prec = WORKLOADS[args.workload]
    p = abi.make_params(content, L=L, precision=prec)
    V = p.sites()
    seed = 20261203 + rank
    f = hot_fields(p, seed)
    lat = gpu.Lattice(p, seed=seed, chain=rank)
    lat.upload(**f)
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
    dev_ms = float(np.sum(step_ms))
    t = torch.tensor([dev_ms], dtype=torch.float64, device=dev)
    if dist:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dev_ms = float(t.item())
    value = world * V * K / (dev_ms * 1e-3)
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
    alg_bytes = REALS_PER_SITE.get(top, 18) * rsize * V
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
    if rank == 0:
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

    # the plain FP64 sweep on the same lattice (the metric's comparison)
    fp64 = None
    if rank == 0 and prec == 32 and not args.no_fp64:
        p64 = abi.make_params(content, L=L, precision=64)
        lat64 = gpu.Lattice(p64, seed=seed)
        lat64.upload(**f)
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
                       "recipe": "1 link heatbath + 4 doublet overrelax + 1 doublet Metropolis, measure each sweep",
                       "couplings": {"betasu2": p.betasu2, "msq": p.msq_phi, "lambda": p.lambda_phi},
                       "reunitarize_interval": p.reunitarize_interval if prec == 32 else None,
                       "l2": "flushed between steps (256 MiB write outside the step events)",
                       "parallelism": f"replicas x{world}", "graph": True,
                       "launch_variants": [int(v) for v in variants]},
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "fp64_plain": fp64,
            # per step: the sweep's kernels, the sweep-counter set/increment, measure + reduction
            "gpu_launches": int(K * (launches_sweep + 4)),
            "clocks": clk, "wall_s_timed_region": t_wall,
            "step_ms_p50": float(np.percentile(step_ms, 50)), "step_ms_p99": float(np.percentile(step_ms, 99)),
        }
        print(json.dumps(line), flush=True)
    lat.close()
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="fund128_f32", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
