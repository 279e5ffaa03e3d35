"""The roofline arithmetic of bench.py (no GPU): algorithmic bytes per launch
from the reals each pass kind touches per site, over the launch time, against
the measured copy bandwidth."""
import importlib.util
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def one_sweep_kinds(nsweeps=1):
    # 6 link half-passes (kind 0), 10 triplet half-passes (kind 3) per sweep
    return np.array(([0] * 6 + [3] * 10) * nsweeps)


def test_persistent_roofline_bytes_and_fraction(bench):
    sites, S = 11011520, 10
    peak, _ = bench.measured_peaks()
    r = bench.persistent_roofline(one_sweep_kinds(3), [25.0, 24.0, 26.0], S, "adj", 32, sites, "no_such_workload",
                                  step_ms=26.0)
    per_sweep = (6 * 17 + 10 * 16.5) * 4 * sites
    assert r["algorithmic_bytes_per_launch"] == pytest.approx(per_sweep * S)
    assert r["avg_launch_ms"] == 25.0  # the median launch
    assert r["achieved"] == pytest.approx(per_sweep * S / 25e-3 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / peak)
    assert r["time_share"] == pytest.approx(25.0 / 26.0)
    assert r["traffic"] is None  # no traffic file for this workload name


def test_persistent_roofline_reads_traffic_per_sweep(bench):
    r = bench.persistent_roofline(one_sweep_kinds(), [24.0], 10, "adj", 32, 11011520, "batched384_adj_f32",
                                  step_ms=27.0)
    # the committed ncu traffic of one sweep, times the sweeps of a launch
    assert r["traffic"] is not None and r["traffic"] > 10 * 0.9 * (6 * 17 + 10 * 16.5) * 4 * 11011520


def test_grouped_roofline_uses_the_grouped_traffic(bench):
    # the grouped sweep: the same algorithmic bytes over the fork-to-join time,
    # the DRAM traffic ncu measured for one grouped sweep (its groups' fields
    # stay in L2 across their passes: far below the algorithmic bytes)
    sites, S = 11011520, 10
    r = bench.persistent_roofline(one_sweep_kinds(), [21.8], S, "adj", 32, sites, "batched384_adj_f32",
                                  step_ms=22.5, groups=(48, 4))
    per_sweep = (6 * 17 + 10 * 16.5) * 4 * sites
    assert r["algorithmic_bytes_per_launch"] == pytest.approx(per_sweep * S)
    assert "48 groups on 4 streams" in r["kernel"]
    assert r["traffic"] is not None and r["traffic"] < 0.2 * per_sweep * S
    p = bench.persistent_roofline(one_sweep_kinds(), [21.8], S, "adj", 32, sites, "batched384_adj_f32",
                                  step_ms=22.5)
    assert p["traffic"] > r["traffic"] and "k_pool_persist" in p["kernel"]


def test_per_pass_roofline_picks_the_largest_share(bench):
    kinds = one_sweep_kinds(2)
    ms = np.where(kinds == 0, 0.18, 0.16)
    r = bench.roofline_of(kinds, ms, "adj", 32, 1000, "no_such_workload")
    assert r["kernel"] == "triplet_update"
    assert r["algorithmic_bytes_per_launch"] == pytest.approx(16.5 * 4 * 1000)
    assert r["avg_launch_ms"] == pytest.approx(0.16)
    assert sum(r["shares"].values()) == pytest.approx(1.0)


def test_sweep_roofline_counts_the_measurement_at_its_cadence(bench):
    # adjoint FP32: 6 x 17 + 10 x 16.5 = 267 reals per sweep, 15 per measurement
    peak, _ = bench.measured_peaks()
    every = bench.sweep_roofline(1e9, "adj", 32)
    per10 = bench.sweep_roofline(1e9, "adj", 32, sweeps_per_measure=10)
    assert every["bytes_per_site_update"] == pytest.approx((267 + 15) * 4)
    assert per10["bytes_per_site_update"] == pytest.approx((267 + 1.5) * 4)
    assert per10["frac"] == pytest.approx(1e9 * 1074 / 1e9 / peak)


def test_batched_config_is_the_same_on_both_arms(bench):
    from su2higgs_gb300 import workloads
    a = bench.batched_config("batched384_adj_f32", workloads.batched_ensemble(384))
    b = bench.batched_config("batched384_adj_f32", workloads.batched_ensemble(384, precision=64))
    assert a == b
    assert a["chains"] == 384 and a["sites_total"] == 11011520
