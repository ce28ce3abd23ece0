"""Beam(file=) and Beam.print_to on the device path against the reference's
own Beam(file) and PrintToFile (goldens from tests/golden/make_beam_files.py)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
Z = np.load(os.path.join(HERE, "golden", "beam_files.npz"))


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_beam_from_file_matches_reference(tmp_path, precision):
    from hpsim_gb300 import HPSim
    f = tmp_path / "quirks.txt"
    f.write_text(str(Z["quirks_text"]))
    beam = HPSim.Beam(file=str(f), precision=precision)
    sc = Z["quirks_scalars"]
    assert beam.get_size() == Z["quirks_cols"].shape[1]
    assert (beam.get_mass(), beam.get_charge(), beam.get_frequency()) == (sc[0], sc[1], sc[3])
    rtol = 0.0 if precision == "fp64" else 1e-6
    for k, name in enumerate(("x", "xp", "y", "yp", "phi", "w")):
        got = beam._coord(name)
        assert np.allclose(got, Z["quirks_cols"][k], rtol=rtol, atol=1e-9 if rtol else 0.0), name
    assert np.array_equal(beam._loss(0), Z["quirks_loss"])
    assert np.array_equal(beam._loss(1), Z["quirks_lloss"])


def test_print_to_is_byte_identical_to_reference(tmp_path):
    from hpsim_gb300 import HPSim
    cols = Z["print_cols"]
    beam = HPSim.Beam(mass=939.294, charge=-1.0, current=0.015, num=cols.shape[1])
    beam.set_distribution(*cols, Z["print_loss"], Z["print_lloss"])
    beam.set_frequency(201.25)
    out = tmp_path / "beam.txt"
    beam.print_to(str(out), "golden beam")
    assert out.read_text() == str(Z["print_text"])


def test_print_then_read_round_trip(tmp_path):
    from hpsim_gb300 import HPSim, lattices as L
    beam = HPSim.Beam(mass=939.294, charge=-1.0, current=0.015, num=4096)
    beam.set_waterbag(*L.waterbag_twiss(), 0.0, 0.75, 201.25, 5)
    out = tmp_path / "wb.txt"
    beam.print_to(str(out), "waterbag")
    back = HPSim.Beam(file=str(out))
    for name in ("x", "xp", "y", "yp", "phi", "w"):
        assert np.allclose(back._coord(name), beam._coord(name), rtol=1e-14, atol=0.0), name
    assert np.array_equal(back._loss(0), beam._loss(0))
