"""File compatibility of the drop-in program bin/su2 with the reference's own
program, on the CPU (bin/su2 --files-only touches no GPU): the labels file, the
binary lattice file (checkpoint.c:84-214) and the multicanonical weight file
(multicanonical.c:82-288) it writes from the reference's inputs are the ones
the reference writes, byte for byte (the two wall-clock doubles of the lattice
header excepted)."""
import os
import struct
import subprocess

import numpy as np
import pytest

import e2e_util as E


@pytest.fixture(scope="module")
def binary():
    return E.ensure_binary()


@pytest.mark.parametrize("case", E.CASES)
def test_labels_lattice_weight_roundtrip(binary, case, tmp_path):
    g = E.stage(case, str(tmp_path))
    E.run(str(tmp_path), g["bin_content"], "--files-only")
    assert E.read(str(tmp_path), "labels") == g["labels"]
    for extra in ("labels_local", "labels_z", "labels_correl"):
        if extra in g:
            assert E.read(str(tmp_path), extra) == g[extra]
    assert E.lattice_equal(E.read(str(tmp_path), "lattice"), g["lattice_out0"])
    if "weight" in g:
        assert E.read(str(tmp_path), "weight") == g["weight"]
    if "in_weight" in g:  # a read-only weight is left as it was (save_weight, multicanonical.c:85-87)
        assert E.read(str(tmp_path), "weight") == g["in_weight"]


def test_cold_start_header(binary, tmp_path):
    """No lattice file: a cold configuration (init.c:92-112) written with
    iteration 1, as a reset run of 0 iterations would."""
    import struct
    g = E.load_case("fund")
    (tmp_path / "config").write_bytes(g["config"])
    E.run(str(tmp_path), "fund", "--files-only")
    data = E.read(str(tmp_path), "lattice")
    size, dim, l1, l2, l3, it = struct.unpack("<5iq", data[:28])
    assert (size, dim, (l1, l2, l3), it) == (1, 3, (6, 4, 8), 1)
    assert len(data) == len(g["lattice_out0"])


def _serial_index(L):
    """storage index of the serial layout (layout.c:657-704) of every
    lexicographic index"""
    V = L[0] * L[1] * L[2]
    n = np.arange(V)
    par = (n % L[0] + (n // L[0]) % L[1] + n // (L[0] * L[1])) % 2
    idx = np.empty(V, np.int64)
    idx[par == 0] = np.arange(int(np.sum(par == 0)))
    idx[par == 1] = int(np.sum(par == 0)) + np.arange(int(np.sum(par == 1)))
    return idx


def _mpi_file(serial, L, ranks, order, ncomps):
    """the lattice file an N-rank run writes (write_field, checkpoint.c:226-269)
    for the fields of a serial one: same header but the MPI size, each field
    block in the order of the reference's MPI layout"""
    sidx = _serial_index(L)[order]
    out = bytearray(serial[:44])
    out[0:4] = struct.pack("<i", ranks)
    off = 44
    V = len(order)
    for n in ncomps:
        blk = np.frombuffer(serial[off: off + 8 * V * n], dtype=np.float64).reshape(V, n)
        out += blk[sidx].tobytes()
        off += 8 * V * n
    assert off == len(serial)
    return bytes(out)


NCOMPS = {"fund": (12, 4), "adj": (12, 3), "su2u1s": (12, 3, 4, 1)}


@pytest.mark.parametrize("case", ["fund", "adj", "su2u1s"])
@pytest.mark.parametrize("ranks", [2, 3, 4, 6, 8, 12, 16])
def test_lattice_files_of_mpi_runs(binary, case, ranks, tmp_path):
    """A lattice file written by an N-rank run of the reference (its sites in
    the order of the reference's own MPI layout code, tests/golden/
    mpi_layout.npz) is read into the right sites and written back in the same
    layout; with lattice_mpi_size 1 it is converted to the serial file the
    reference writes."""
    g = E.stage(case, str(tmp_path))
    L = (6, 4, 8)
    order = np.load(os.path.join(E.GOLDEN, "mpi_layout.npz"))[f"order_6x4x8_{ranks}"]
    mpi = _mpi_file(g["lattice_in"], L, ranks, order, NCOMPS[case])
    (tmp_path / "lattice").write_bytes(mpi)
    E.run(str(tmp_path), g["bin_content"], "--files-only")
    back = E.read(str(tmp_path), "lattice")
    assert back[:20] == mpi[:20] and back[44:] == mpi[44:]
    (tmp_path / "config").write_bytes(g["config"] + b"\nlattice_mpi_size 1\n")
    E.run(str(tmp_path), g["bin_content"], "--files-only")
    serial = E.read(str(tmp_path), "lattice")
    want = g["lattice_out0"]
    assert serial[:20] == want[:20] and serial[44:] == want[44:]
    # and from the serial file to the N-rank layout
    (tmp_path / "config").write_bytes(g["config"] + f"\nlattice_mpi_size {ranks}\n".encode())
    E.run(str(tmp_path), g["bin_content"], "--files-only")
    again = E.read(str(tmp_path), "lattice")
    assert again[:20] == mpi[:20] and again[44:] == mpi[44:]


def test_lattice_file_of_impossible_rank_count_is_refused(binary, tmp_path):
    """5 ranks cannot share 6x4x8 sites (make_slices, layout.c:118-122): the
    file is refused as the reference refuses a mismatched one."""
    g = E.stage("fund", str(tmp_path))
    data = bytearray(g["lattice_in"])
    data[0:4] = struct.pack("<i", 5)
    (tmp_path / "lattice").write_bytes(bytes(data))
    r = subprocess.run([E.BIN, "--content", g["bin_content"], "--files-only", "config"], cwd=str(tmp_path),
                       capture_output=True, text=True, timeout=60)
    assert r.returncode != 0
    assert "do not match" in r.stdout


@pytest.mark.parametrize("L,ranks", [((8, 8, 8), 4), ((10, 6, 12), 15), ((16, 8, 12), 12)])
def test_mpi_layouts_of_other_lattices(binary, L, ranks, tmp_path):
    """The same conversion on other sides and rank counts (slicings 2x2x1,
    5x1x3, 4x1x3 in the reference's layout), with seeded random fields."""
    import re
    g = E.load_case("fund")
    cfg = g["config"].decode()
    for d, n in enumerate(L):
        cfg = re.sub(r"^L%d\s+\S+.*$" % (d + 1), f"L{d + 1} {n}", cfg, flags=re.M)
    (tmp_path / "config").write_text(cfg + "\nlattice_mpi_size 1\n")
    V = L[0] * L[1] * L[2]
    rng = np.random.default_rng(V + ranks)
    serial = struct.pack("<5iqdd", 1, 3, *L, 7, 0.0, 0.0) + rng.normal(size=V * 16).tobytes()
    order = np.load(os.path.join(E.GOLDEN, "mpi_layout.npz"))["order_%s_%d" % ("x".join(map(str, L)), ranks)]
    (tmp_path / "lattice").write_bytes(_mpi_file(serial, L, ranks, order, (12, 4)))
    E.run(str(tmp_path), "fund", "--files-only")
    out = E.read(str(tmp_path), "lattice")
    assert out[:20] == serial[:20] and out[44:] == serial[44:]
