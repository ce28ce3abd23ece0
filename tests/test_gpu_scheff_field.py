"""The SCHEFF table stage through the C ABI (hps_scheff_field) against the
reference's charge table -> field table pair."""
import numpy as np
import pytest

from tests import golden_cases as G

pytestmark = pytest.mark.gpu


def field(nr, nz, bins, mesh):
    from hpsim_gb300._capi import call, dptr
    out = np.zeros((nz + 1) * (nr + 1) * 2)
    call("hps_scheff_field", nr, nz, dptr(np.ascontiguousarray(bins)), dptr(np.ascontiguousarray(mesh)), dptr(out))
    return out


def test_field_table_matches_reference():
    z = np.load(f"{G.GOLDEN}/scheff_tables_8x64.npz")
    f = field(8, 64, z["bin"], z["mesh"])
    ref = z["fld2"]
    assert np.allclose(f, ref, rtol=1e-9, atol=1e-12 * np.abs(ref).max())
    assert f[-2:].tolist() == [0.0, 0.0]  # corner left at zero below 1024 bins


def test_field_table_32x128_against_oracle(oracle):
    """A 32x128 mesh with adjacent-bunch images, random charges."""
    import ctypes as C
    rng = np.random.default_rng(3)
    nr, nz = 32, 128
    bins = rng.uniform(0.0, 5.0, nr * nz) * (rng.uniform(size=nr * nz) > 0.3)
    mesh = np.array([4.0e-4, 2.0e-4, 0.05, 201.25, 65536, 1.6e-5, 2.0])
    f = field(nr, nz, bins, mesh)
    s = oracle.Scheff(nr, nz, 0.01, 0)
    s.s.dr, s.s.dz = mesh[0], mesh[1]
    oracle.lib().orc_scheff_green_table(s.h, mesh[2], mesh[3], int(mesh[4]), mesh[5], int(mesh[6]))
    C.memmove(s.s.bin, bins.ctypes.data, bins.nbytes)
    oracle.lib().orc_scheff_contract(s.h)
    _, _, ref = s.tables()
    assert np.allclose(f, ref, rtol=1e-9, atol=1e-12 * np.abs(ref).max())
