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


def field_f32(nr, nz, bins, mesh):
    from hpsim_gb300._capi import call, dptr
    out = np.zeros((nz + 1) * (nr + 1) * 2)
    call("hps_scheff_field_f32", nr, nz, dptr(np.ascontiguousarray(bins)), dptr(np.ascontiguousarray(mesh)),
         dptr(out))
    return out


def _close_per_component(f, ref, tol):
    """|error| <= tol * max|E| for E_r and E_z separately."""
    for c in (0, 1):
        a, b = f[c::2], ref[c::2]
        assert np.max(np.abs(a - b)) <= tol * np.max(np.abs(b)), (c, np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_field_f32_matches_reference():
    """FP32 Green's table and contraction against the reference's FP64
    charge -> field pair: |error| <= 2e-5 of the largest field component."""
    z = np.load(f"{G.GOLDEN}/scheff_tables_8x64.npz")
    f = field_f32(8, 64, z["bin"], z["mesh"])
    _close_per_component(f, z["fld2"], 2e-5)
    assert f[-2:].tolist() == [0.0, 0.0]


@pytest.mark.parametrize("adj", [0, 2])
def test_field_f32_32x128_against_fp64(adj):
    """A bunched (Gaussian in r and z) charge table on 32 x 128, with and
    without adjacent-bunch images: FP32 table stage within 2e-5 of the
    largest component of the FP64 one."""
    nr, nz = 32, 128
    r = (np.arange(nr) + 0.5) / nr
    zz = (np.arange(nz) + 0.5) / nz - 0.5
    q = np.exp(-(zz[:, None] / 0.15) ** 2 - (r[None, :] / 0.3) ** 2) * 2 * np.pi * r[None, :] * 5000
    bins = np.round(q * 2 ** 20) / 2 ** 20
    mesh = np.array([4.0e-4, 2.0e-4, 0.05, 201.25, 65536, 1.6e-5, float(adj)])
    _close_per_component(field_f32(nr, nz, bins.ravel(), mesh), field(nr, nz, bins.ravel(), mesh), 2e-5)


def test_field_f32_64x256_against_fp64():
    """The 64 x 256 mesh of the CCL workloads (32-radius tiles of the
    single-copy table, four row slabs per block): FP32 table stage within 2e-5
    of the largest component of the FP64 one."""
    nr, nz = 64, 256
    r = (np.arange(nr) + 0.5) / nr
    zz = (np.arange(nz) + 0.5) / nz - 0.5
    q = np.exp(-(zz[:, None] / 0.12) ** 2 - (r[None, :] / 0.25) ** 2) * 2 * np.pi * r[None, :] * 5000
    bins = np.round(q * 2 ** 20) / 2 ** 20
    mesh = np.array([2.0e-4, 1.0e-4, 0.43, 805.0, 1048576, 1.6e-5, 0.0])
    _close_per_component(field_f32(nr, nz, bins.ravel(), mesh), field(nr, nz, bins.ravel(), mesh), 2e-5)


def test_field_table_64x256_against_oracle(oracle):
    """The 64 x 256 mesh in FP64 (single-copy table tiles of 16 source
    radii): random charges against the oracle's Green's table and
    contraction."""
    import ctypes as C
    rng = np.random.default_rng(4)
    nr, nz = 64, 256
    bins = np.ascontiguousarray(rng.uniform(0.0, 5.0, nr * nz) * (rng.uniform(size=nr * nz) > 0.3))
    mesh = np.array([2.0e-4, 1.0e-4, 0.43, 805.0, 1048576, 1.6e-5, 0.0])
    f = field(nr, nz, bins, mesh)
    s = oracle.Scheff(nr, nz, 0.01, 0)
    s.s.dr, s.s.dz = mesh[0], mesh[1]
    oracle.lib().orc_scheff_green_table(s.h, mesh[2], mesh[3], int(mesh[4]), mesh[5], int(mesh[6]))
    C.memmove(s.s.bin, bins.ctypes.data, bins.nbytes)
    oracle.lib().orc_scheff_contract(s.h)
    _, _, ref = s.tables()
    assert np.allclose(f, ref, rtol=1e-9, atol=1e-12 * np.abs(ref).max())


def field_f32_kernel(nr, nz, bins, mesh, kernel):
    from hpsim_gb300._capi import call, dptr
    out = np.zeros((nz + 1) * (nr + 1) * 2)
    call("hps_scheff_field_f32_kernel", nr, nz, dptr(np.ascontiguousarray(bins)), dptr(np.ascontiguousarray(mesh)),
         dptr(out), kernel)
    return out


def _bunched(nr, nz, sz=0.12, sr=0.25):
    r = (np.arange(nr) + 0.5) / nr
    zz = (np.arange(nz) + 0.5) / nz - 0.5
    q = np.exp(-(zz[:, None] / sz) ** 2 - (r[None, :] / sr) ** 2) * 2 * np.pi * r[None, :] * 5000
    return (np.round(q * 2 ** 20) / 2 ** 20).ravel()


@pytest.mark.parametrize("nr,nz", [(16, 128), (32, 128), (32, 256), (64, 256), (16, 512), (64, 512)])
def test_tensor_core_contraction_against_fp64(nr, nz):
    """The split-BF16 tcgen05 contraction (kernel 2) on bunched and random
    charge tables: within 2e-5 of the largest field component of the FP64
    table stage, and within 2e-5 of the FP32 CUDA-core contraction (kernel
    1), on every mesh shape the tensor-core path takes."""
    mesh = np.array([2.0e-4, 1.0e-4, 0.43, 805.0, 1048576, 1.6e-5, 0.0])
    rng = np.random.default_rng(nr + nz)
    for bins in (_bunched(nr, nz), rng.uniform(0.0, 5.0, nr * nz) * (rng.uniform(size=nr * nz) > 0.3)):
        tc = field_f32_kernel(nr, nz, bins, mesh, 2)
        cuda = field_f32_kernel(nr, nz, bins, mesh, 1)
        _close_per_component(tc, field(nr, nz, bins, mesh), 2e-5)
        _close_per_component(tc, cuda, 2e-5)
        assert np.array_equal(tc, field_f32_kernel(nr, nz, bins, mesh, 2))  # deterministic


def test_tensor_core_contraction_adjacent_bunches():
    """32 x 128 with adjacent-bunch images in the Green's table."""
    nr, nz = 32, 128
    mesh = np.array([4.0e-4, 2.0e-4, 0.05, 201.25, 65536, 1.6e-5, 2.0])
    bins = _bunched(nr, nz, 0.15, 0.3)
    _close_per_component(field_f32_kernel(nr, nz, bins, mesh, 2), field(nr, nz, bins, mesh), 2e-5)


def test_tensor_core_contraction_rejects_other_meshes():
    from hpsim_gb300._capi import HPSimError
    mesh = np.array([2.0e-4, 1.0e-4, 0.43, 805.0, 1048576, 1.6e-5, 0.0])
    for nr, nz in ((8, 64), (8, 128), (32, 64), (128, 256)):
        with pytest.raises(HPSimError):
            field_f32_kernel(nr, nz, np.ones(nr * nz), mesh, 2)
        # the default kernel takes the FP32 ring convolution there
        _close_per_component(field_f32_kernel(nr, nz, np.ones(nr * nz), mesh, 0),
                             field(nr, nz, np.ones(nr * nz), mesh), 2e-5)
