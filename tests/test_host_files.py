"""File compatibility of the drop-in program bin/su2 with the reference's own
program, on the CPU (bin/su2 --files-only touches no GPU): the labels file, the
binary lattice file (checkpoint.c:84-214) and the multicanonical weight file
(multicanonical.c:82-288) it writes from the reference's inputs are the ones
the reference writes, byte for byte (the two wall-clock doubles of the lattice
header excepted)."""
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
