"""Shared helpers of the bin/su2 drop-in tests: the golden runs of the
reference's own program (tests/golden/e2e_<case>.npz, made by
tests/golden/make_e2e.py) replayed through bin/su2 in scratch directories."""
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
BIN = os.path.join(ROOT, "bin", "su2")
CASES = ("fund", "adj", "su2u1s", "fund_muca", "su2u1s_z", "fundadj_z", "fund_traj", "adj_corr", "fundadj_corr")


def ensure_binary():
    """bin/su2 (and the library it links) built from this checkout."""
    lib = os.path.join(ROOT, "su2higgs_gb300", "libsu2gpu.so")
    if not os.path.exists(lib):
        from su2higgs_gb300 import build
        build.build()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "su2higgs_gb300", "host")], check=True)
    return BIN


def load_case(case):
    """The golden run; "bin_content" is the field content to give bin/su2
    (the -D flags the reference binary was built with)."""
    d = np.load(os.path.join(GOLDEN, f"e2e_{case}.npz"))
    return {k: (str(d[k]) if k in ("content", "bin_content") else bytes(d[k])) for k in d.files}


def stage(case, tmpdir):
    g = load_case(case)
    with open(os.path.join(tmpdir, "config"), "wb") as f:
        f.write(g["config"])
    with open(os.path.join(tmpdir, "lattice"), "wb") as f:
        f.write(g["lattice_in"])
    if "weight" in g:
        with open(os.path.join(tmpdir, "weight"), "wb") as f:
            f.write(g["weight"])
    # further inputs of the case (in_<file name>)
    for k in g:
        if k.startswith("in_"):
            with open(os.path.join(tmpdir, k[3:]), "wb") as f:
                f.write(g[k])
    return g


def run(tmpdir, content, *args, timeout=600):
    r = subprocess.run([BIN, "--content", content, *args, "config"], cwd=tmpdir, capture_output=True, text=True,
                       timeout=timeout)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    return r.stdout


def read(tmpdir, name):
    with open(os.path.join(tmpdir, name), "rb") as f:
        return f.read()


def lattice_equal(a, b):
    """Equal lattice files: header (MPI size, dim, L, iteration) and fields;
    the two time doubles after the iteration counter are not compared."""
    return len(a) == len(b) and a[:28] == b[:28] and a[44:] == b[44:]
