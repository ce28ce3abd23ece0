"""Beam text files (hpsim_gb300/beam_io.py) against the reference's own
Beam::PrintToFile and Beam(file) (goldens from tests/golden/make_beam_files.py,
which runs the reference's Beam class compiled for the host)."""
import os

import numpy as np

from hpsim_gb300 import beam_io as B

HERE = os.path.dirname(os.path.abspath(__file__))
Z = np.load(os.path.join(HERE, "golden", "beam_files.npz"))


def test_writer_is_byte_identical_to_the_reference(tmp_path):
    cols = [c.copy() for c in Z["print_cols"]]
    for k in range(4):  # InitBeamFromDistribution puts particle 0 on axis
        cols[k][0] = 0.0
    out = tmp_path / "beam.txt"
    B.write_beam_file(str(out), "golden beam", -1.0, 939.294, 0.015, 201.25, cols, Z["print_loss"],
                      Z["print_lloss"])
    assert out.read_text() == str(Z["print_text"])


def test_reader_follows_the_reference_on_corner_cases(tmp_path):
    f = tmp_path / "quirks.txt"
    f.write_text(str(Z["quirks_text"]))
    mass, charge, current, freq, cols = B.read_beam_file(str(f))
    sc = Z["quirks_scalars"]
    assert (mass, charge, current, freq) == tuple(sc[:4])  # current 1.5: no exponents in header values
    assert len(cols[0]) == Z["quirks_cols"].shape[1] == 4   # tab and '+' lines are not particle lines
    for k in range(6):
        assert np.array_equal(cols[k], Z["quirks_cols"][k]), k
    assert np.array_equal(cols[6], Z["quirks_loss"]) and np.array_equal(cols[7], Z["quirks_lloss"])
    assert cols[5][0] == sc[4]  # design energy = w of particle 0


def test_round_trip_keeps_15_significant_digits(tmp_path):
    rng = np.random.default_rng(11)
    n = 1000
    cols = [rng.normal(scale=s, size=n) for s in (1e-3, 2e-3, 1e-3, 2e-3, 0.3)] + [0.75 + 0.01 * rng.random(n)]
    for k in range(4):
        cols[k][0] = 0.0
    loss = rng.integers(0, 400, n).astype(np.uint32) * (rng.random(n) < 0.1)
    lloss = (rng.random(n) < 0.05).astype(np.uint32)
    f = tmp_path / "rt.txt"
    B.write_beam_file(str(f), "round trip", -1.0, 939.294, 0.015, 201.25, cols, loss, lloss)
    mass, charge, current, freq, back = B.read_beam_file(str(f))
    assert (mass, charge, current, freq) == (939.294, -1.0, 0.015, 201.25)
    for k in range(6):
        assert np.allclose(back[k], cols[k], rtol=1e-14, atol=0.0), k
    assert np.array_equal(back[6], loss) and np.array_equal(back[7], lloss)


def test_six_columns_give_no_loss_arrays(tmp_path):
    f = tmp_path / "six.txt"
    f.write_text("Charge -1\nMass 939.294\nCurrent 0\nFrequency 201.25\n0 0 0 0 0 0.75\n1e-3 0 0 0 0.1 0.76\n")
    *_, cols = B.read_beam_file(str(f))
    assert cols[6] is None and cols[7] is None and cols[5][1] == 0.76


def test_missing_header_value_raises(tmp_path):
    f = tmp_path / "bad.txt"
    f.write_text("Charge -1\nMass 939.294\nFrequency 201.25\n0 0 0 0 0 0.75\n")
    try:
        B.read_beam_file(str(f))
    except ValueError as e:
        assert "current" in str(e)
    else:
        raise AssertionError("no error for a file without a current")
