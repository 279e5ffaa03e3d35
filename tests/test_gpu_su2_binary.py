"""bin/su2, the drop-in for the reference's program, against the reference's
own outputs (tests/golden/e2e_<case>.npz): from the same config and lattice
file, with reset 0, the first measure row and the first measure_flow block are
taken on the loaded configuration before any update (main.c:306-318), so
they are deterministic.  Checked: the labels file byte for byte, the same
number of columns and lines, every printed value within the stated tolerance
of the reference's (FP64 path: 1e-6 relative -- six printed digits, so equal
up to the rounding of the last printed digit; FP32 form: 1e-4 relative,
1e-5 absolute), the measure_local files of the flow (coordinates exact, the
values within the same tolerances), and the lattice file the run leaves
behind is a valid checkpoint of the right size that bin/su2 reads back."""
import numpy as np
import pytest

import e2e_util as E

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def binary():
    return E.ensure_binary()


def rows(text):
    return [line.split() for line in text.decode().splitlines() if line.strip()]


def close(a, b, rtol, atol):
    x, y = float(a), float(b)
    return abs(x - y) <= atol + rtol * max(abs(x), abs(y))


def compare_rows(got, want, rtol, atol):
    assert len(got) == len(want), (got, want)
    for rg, rw in zip(got, want):
        if rg[0].startswith("="):
            assert rg == rw
            continue
        assert len(rg) == len(rw), (rg, rw)
        for a, b in zip(rg, rw):
            assert close(a, b, rtol, atol), (a, b, rg, rw)


@pytest.mark.parametrize("precision,rtol,atol", [(64, 1e-6, 1e-12), (32, 1e-4, 1e-5)])
@pytest.mark.parametrize("case", ["fund", "adj", "su2u1s"])
def test_first_measurement_and_flow_match_reference(binary, case, precision, rtol, atol, tmp_path):
    d = str(tmp_path)
    g = E.stage(case, d)
    E.run(d, g["bin_content"], "--precision", str(precision), "--seed", "7")
    assert E.read(d, "labels") == g["labels"]
    got = rows(E.read(d, "measure"))
    want = rows(g["measure"])
    assert len(got) == len(want) == 1
    compare_rows(got, want, rtol, atol)
    if precision == 64:
        # FP64: the printed row is the reference's except in a last-digit
        # rounding case
        same = sum(a == b for a, b in zip(got[0], want[0]))
        assert same >= len(want[0]) - 1, (got, want)
    compare_rows(rows(E.read(d, "measure_flow")), rows(g["measure_flow"]), rtol, atol)
    # measure_local files of the flow (binary: 3 ints of coordinates, with the
    # triplet Tr Sigma^2 and the charge as doubles, a newline byte per site)
    local = sorted(k for k in g if k.startswith("measure_local_"))
    if local:
        assert E.read(d, "labels_local") == g["labels_local"]
        has_t = g["content"] in ("adj", "fundadj")
        dt = np.dtype([("c", "<i4", 3)] + ([("v", "<f8", 2)] if has_t else []) + [("nl", "u1")])
        for name in local:
            a = np.frombuffer(E.read(d, name), dtype=dt)
            b = np.frombuffer(g[name], dtype=dt)
            assert len(a) == len(b) and np.array_equal(a["c"], b["c"]) and np.all(a["nl"] == 10), name
            if has_t:
                assert np.allclose(a["v"][:, 0], b["v"][:, 0], rtol=rtol, atol=atol), name
                assert np.max(np.abs(a["v"][:, 1] - b["v"][:, 1])) < (1e-9 if precision == 64 else 1e-3), name
    out = E.read(d, "lattice")
    assert len(out) == len(g["lattice_in"])
    assert out[:20] == g["lattice_in"][:20]
    # the checkpoint it wrote is read back (a run of 0 iterations keeps it)
    E.run(d, g["bin_content"], "--files-only")
    again = E.read(d, "lattice")
    assert again[44:] == out[44:]


@pytest.mark.parametrize("precision,rtol,atol", [(64, 1e-6, 1e-12), (32, 1e-4, 1e-5)])
@pytest.mark.parametrize("case", ["su2u1s_z", "fundadj_z"])
def test_first_z_profile_matches_reference(binary, case, precision, rtol, atol, tmp_path):
    """Profiles along z (the reference's -DMEASURE_Z build): labels_z byte for
    byte, and the first measure_z block -- plane averages of the loaded
    configuration, taken before the first update -- value by value."""
    d = str(tmp_path)
    g = E.stage(case, d)
    E.run(d, g["bin_content"], "--precision", str(precision), "--seed", "7")
    assert E.read(d, "labels") == g["labels"]
    assert E.read(d, "labels_z") == g["labels_z"]
    compare_rows(rows(E.read(d, "measure")), rows(g["measure"]), rtol, atol)
    compare_rows(rows(E.read(d, "measure_z")), rows(g["measure_z"]), rtol, atol)


def _realtime_band(g):
    kv = dict(line.split()[:2] for line in g["in_realtime_config"].decode().splitlines() if line.strip())
    return float(kv["min"]), float(kv["max"]), int(kv["n_traj"])


@pytest.mark.parametrize("precision,tol", [(64, 1e-7), (32, 1e-5)])
def test_trajectories_match_reference(binary, precision, tol, tmp_path):
    """Heatbath trajectories (the reference's -DHB_TRAJECTORY build,
    hb_trajectory.c:10-94): the trajectory file has the reference's lines --
    run header, set header with the start value, one header per trajectory,
    "sweeps value" rows -- and each trajectory starts at the order parameter
    of the loaded configuration (within `tol`) and ends, in the band of
    +-1e-4 around it, after its first sweep with a value outside the band
    (the value itself is random).  The main run is unchanged by the
    trajectories: its first measure row is the reference's."""
    d = str(tmp_path)
    g = E.stage("fund_traj", d)
    E.run(d, g["bin_content"], "--precision", str(precision), "--seed", "7")
    lo, hi, n = _realtime_band(g)
    got = E.read(d, "trajectory").decode().splitlines()
    want = g["trajectory"].decode().splitlines()
    assert len(got) == len(want)
    starts = 0
    for a, b in zip(got, want):
        if not b.strip() or b.startswith("=") or b.startswith("--- Traj"):
            assert a == b
        elif b.startswith("----- Begin set"):
            pa, pb = a.split(), b.split()
            assert pa[:6] == pb[:6] and pa[7:] == pb[7:]
            assert close(pa[6], pb[6], 1e-6 if precision == 64 else 1e-5, tol)
        else:
            (ia, va), (ib, vb) = a.split(), b.split()
            assert ia == ib
            if ib == "0":
                starts += 1
                assert close(va, vb, 0.0, tol)
            else:
                assert float(va) < lo or float(va) > hi
                assert len(va.split(".")[1]) == 8
    assert starts == n
    compare_rows(rows(E.read(d, "measure")), rows(g["measure"]), 1e-6 if precision == 64 else 1e-4, 1e-5)


@pytest.mark.parametrize("precision,rtol,atol", [(64, 1e-6, 1e-12), (32, 1e-4, 1e-5)])
@pytest.mark.parametrize("case", ["adj_corr", "fundadj_corr"])
def test_first_correlators_match_reference(binary, case, precision, rtol, atol, tmp_path):
    """Correlators (the reference's -DCORRELATORS -DBLOCKING build):
    labels_correl byte for byte; the first correl0 block -- of the loaded
    configuration, before the first update -- and, without a doublet, the
    first correl1 block of the blocked lattice (6x4x8 -> 3x2x8) value by
    value; with a doublet no blocked file, as the reference writes none."""
    d = str(tmp_path)
    g = E.stage(case, d)
    E.run(d, g["bin_content"], "--precision", str(precision), "--seed", "7")
    assert E.read(d, "labels_correl") == g["labels_correl"]
    for name in ("correl0", "correl1"):
        if name in g:
            got, want = rows(E.read(d, name)), rows(g[name])
            # photon columns whose value is 0 up to rounding (imaginary parts at
            # distance 0) are compared against the column's scale
            compare_rows(got, want, rtol, atol if precision == 64 else 1e-3)
        else:
            import os
            assert not os.path.exists(os.path.join(d, name))
