"""Golden files of the reference program itself (bin/su2 drop-in checks).

Runs the reference's own serial binaries (built from its sources by
`make -C oracle/ref`, outputs in oracle/_ref/su2_<content>) in scratch
directories and stores, per case, in e2e_<case>.npz:

  config        the config file (the reference's sample config, main keys set)
  lattice_in    a seeded hot lattice in the reference's binary format
                (checkpoint.c:84-122), iteration counter 0
  labels        the labels file the reference writes (measure.c:15-64)
  measure       its measure file after `iterations 1`: the row of the loaded
                configuration, taken before the first update (main.c:306-310)
  measure_flow  its measure_flow block of the same configuration
                (gradflow.c:66-160), flow before the first update
  labels_local, measure_local_1_<k>
                (fund, adj: measure_local 1) the local-measurement labels and
                the binary per-site files written at every flow measurement
                (measure.c:347-487)
  lattice_out0  the lattice file it writes after `iterations 0` (fields as
                loaded, header iteration 1; the two time doubles are not
                compared)
  weight        (muca case) the weight file the reference wrote during a
                multicanonical run (multicanonical.c:82-111)
  labels_z, measure_z
                (the _z cases, -DMEASURE_Z builds) the profile labels and the
                first measure_along_z block, of the loaded configuration
                (z_coord.c:78-300)
  trajectory    (fund_traj, the -DHB_TRAJECTORY build) the trajectory file of
                one set of heatbath trajectories started at iteration 1 from
                the loaded configuration (hb_trajectory.c:10-94), in a band of
                +-1e-4 around its order parameter so that every trajectory
                ends after one sweep
  labels_correl, correl0, correl1
                (the _corr cases, -DCORRELATORS -DBLOCKING builds) the
                correlator labels and the first correlator blocks of the
                loaded configuration, of the lattice itself and of its
                blocking levels (correlation.c:320-432)
  in_<name>     further input files of the case (flat read-only weight,
                realtime_config), written next to the config before the run
  bin_content   the --content argument that makes bin/su2 the same program

Run here, where the reference sources are: python tests/golden/make_e2e.py
"""
import os
import re
import shutil
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from su2higgs_gb300 import abi, workloads  # noqa: E402

# the reference checkout's example config (SU2HIGGS_REF overrides its location)
REF_CONFIG = os.path.join(os.environ.get("SU2HIGGS_REF", "/root/reference"), "config")
REF_BIN = os.path.join(ROOT, "oracle", "_ref")
L = (6, 4, 8)

CASES = {
    # case: (reference binary, field content, bin/su2 content, config overrides)
    "fund": ("fund", "fund", "fund+gradflow", {"measure_local": 1}),
    "adj": ("adj", "adj", "adj+gradflow", {"measure_local": 1}),
    "su2u1s": ("su2u1s", "su2u1s", "su2u1s+gradflow", {}),
    "fund_muca": ("fund", "fund", "fund+gradflow", {"multicanonical": 1, "muca_mode": 1, "bins": 20, "min": 0.0,
                                                     "max": 0.6, "iterations": 30, "interval": 10, "do_flow": 0}),
    # profiles along z (-DMEASURE_Z builds): the first measure_z block is of
    # the loaded configuration, before any update (main.c:308-311)
    "su2u1s_z": ("su2u1sz", "su2u1s", "su2u1s+measure_z", {"do_flow": 0, "do_z_meas": 1, "interval_z": 1,
                                                          "setup_wall": 0}),
    "fundadj_z": ("fundadjz", "fundadj", "fundadj+measure_z", {"do_flow": 0, "do_z_meas": 1, "interval_z": 1,
                                                               "setup_wall": 0}),
    # heatbath trajectories (-DHB_TRAJECTORY): a read-only flat weight, one
    # set at iteration 1 (mode_interval 1)
    "fund_traj": ("fundt", "fund", "fund+hb_trajectory", {"do_flow": 0, "multicanonical": 1, "muca_mode": 0,
                                                          "bins": 20, "min": 0.0, "max": 1.2, "orderparam": "phisq",
                                                          "do_trajectory": 1}),
    # correlators along the longest direction, blocked once (6x4x8 -> 3x2x8);
    # with a doublet the reference writes no blocked correlators
    "adj_corr": ("adjc", "adj", "adj+correlators+blocking", {"do_flow": 0, "do_correlators": 1,
                                                             "correlator_interval": 1, "blocks": 2}),
    "fundadj_corr": ("fundadjc", "fundadj", "fundadj+correlators+blocking",
                     {"do_flow": 0, "do_correlators": 1, "correlator_interval": 1, "blocks": 2}),
}

TRAJ_BAND = 1e-4
TRAJ_N = 3


def flat_weight(bins=20, lo=0.0, hi=1.2):
    """A flat weight file in the reference's format (save_weight,
    multicanonical.c:82-99): bins delta last_max wrk_min wrk_max, then the
    bins+1 bin starts with weight 0."""
    lines = ["%d %.12f %d %f %f" % (bins, 0.3, 0, lo, hi)]
    for i in range(bins + 1):
        lines.append("%f %f" % (lo + i * (hi - lo) / bins, 0.0))
    return ("\n".join(lines) + "\n").encode()


def phisq(content, lat):
    """calc_orderparam PHISQ (multicanonical.c:709-749) of a lattice file:
    sum of |phi|^2 / 2 over the EVEN then the ODD sites, each divided by the
    volume."""
    V = L[0] * L[1] * L[2]
    off = 44 + 8 * V * 3 * 4
    phi = np.frombuffer(lat[off:off + 8 * V * 4], dtype=np.float64).reshape(V, 4)
    sq = 0.5 * np.sum(phi * phi, axis=1)
    return float(np.sum(sq[: V // 2]) / V + np.sum(sq[V // 2:]) / V)


def extra_inputs(case, content, lat):
    if case != "fund_traj":
        return {}
    v0 = phisq(content, lat)
    rt = "n_traj %d\ninterval 1\nmode_interval 1\nmin %.10f\nmax %.10f\n" % (TRAJ_N, v0 - TRAJ_BAND,
                                                                              v0 + TRAJ_BAND)
    return {"weight": flat_weight(), "realtime_config": rt.encode()}


def set_key(text, key, value):
    pat = re.compile(r"^%s\s+\S+.*$" % re.escape(key), re.M)
    if pat.search(text):
        return pat.sub(lambda m: f"{key} {value}", text, count=1)
    return text + f"\n{key} {value}\n"


def make_config(over):
    text = open(REF_CONFIG).read()
    base = dict(L1=L[0], L2=L[1], L3=L[2], reset=0, iterations=1, n_thermalize=0, interval=1, checkpoint=1000,
                run_checks=0, multicanonical=0, do_flow=1, flow_interval=1, flow_t_max=0.1, flow_dt=0.02,
                flow_meas_interval=2, do_z_meas=0, setup_wall=0, scalar_sweeps=4, do_correlators=0,
                measure_local=0)
    base.update(over)
    for k, v in base.items():
        text = set_key(text, k, v)
    return text


def lattice_bytes(content, seed, it=0):
    p = abi.make_params(content, L=L)
    f = workloads.hot_fields(p, seed, phi_sigma=0.5, trip_sigma=0.4, sing_sigma=0.4)
    out = struct.pack("ii", 1, 3) + struct.pack("iii", *L) + struct.pack("ldd", it, 0.0, 0.0)
    for n in ("link", "u1", "d0", "d1", "trip", "sing"):
        if n in f:
            out += np.ascontiguousarray(f[n], dtype=np.float64).tobytes()
    return out


def run_ref(content, config, lattice, extra=None):
    d = tempfile.mkdtemp()
    try:
        open(os.path.join(d, "config"), "w").write(config)
        open(os.path.join(d, "lattice"), "wb").write(lattice)
        if extra:
            for name, data in extra.items():
                open(os.path.join(d, name), "wb").write(data)
        r = subprocess.run([os.path.join(REF_BIN, "su2_" + content), "config"], cwd=d, capture_output=True,
                           text=True, timeout=600)
        if r.returncode != 0:
            raise RuntimeError(r.stdout[-2000:] + r.stderr[-2000:])
        out = {}
        for name in sorted(os.listdir(d)):
            if name in ("labels", "measure", "measure_flow", "lattice", "weight", "labels_local", "labels_z",
                        "measure_z", "trajectory", "labels_correl") or name.startswith("measure_local_") \
                    or name.startswith("correl"):
                out[name] = open(os.path.join(d, name), "rb").read()
        return out
    finally:
        shutil.rmtree(d)


def main(only=None):
    for case, (binary, content, bin_content, over) in CASES.items():
        if only and case not in only:
            continue
        config = make_config(over)
        lat = lattice_bytes(content, 1000 + len(case))
        extra = extra_inputs(case, content, lat)
        got = run_ref(binary, config, lat, extra)
        rec = {"config": np.frombuffer(config.encode(), dtype=np.uint8), "content": np.array(content),
               "bin_content": np.array(bin_content),
               "lattice_in": np.frombuffer(lat, dtype=np.uint8),
               "labels": np.frombuffer(got["labels"], dtype=np.uint8),
               "measure": np.frombuffer(got["measure"], dtype=np.uint8)}
        if "measure_flow" in got:
            rec["measure_flow"] = np.frombuffer(got["measure_flow"], dtype=np.uint8)
        if "weight" in got and "weight" not in extra:
            rec["weight"] = np.frombuffer(got["weight"], dtype=np.uint8)
        for name, data in extra.items():
            rec["in_" + name] = np.frombuffer(data, dtype=np.uint8)
        for name, data in got.items():
            if name in ("labels_local", "labels_z", "measure_z", "trajectory", "labels_correl") or \
                    name.startswith("measure_local_") or name.startswith("correl"):
                rec[name] = np.frombuffer(data, dtype=np.uint8)
        got0 = run_ref(binary, set_key(config, "iterations", 0), lat, extra)
        rec["lattice_out0"] = np.frombuffer(got0["lattice"], dtype=np.uint8)
        np.savez_compressed(os.path.join(HERE, f"e2e_{case}.npz"), **rec)
        print(case, {k: len(v) for k, v in got.items()})


if __name__ == "__main__":
    main(sys.argv[1:])
