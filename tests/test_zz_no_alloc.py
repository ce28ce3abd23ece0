"""hps_scheff_field_noalloc: the SCHEFF field solve for callers that must not
allocate device memory while they run (an online model inside a control
cycle, a host that owns the device through its own memory pool).

The entry point keeps its intermediate tables in a static device array of
the library instead of allocating them; the caller passes the charge table
and receives the field table in its own device buffers.  Its results must
equal those of the allocating entry point hps_scheff_field, call after call
(the static scratch keeps the previous call's contents).  This file is
collected last so that a failure here leaves every other test already run.
"""
import os
import re

import numpy as np
import pytest

from tests.conftest import ROOT

HPS_ERR_INVALID = 1


def _allocating(nr, nz, bins, mesh):
    from hpsim_gb300._capi import call, dptr
    out = np.zeros((nz + 1) * (nr + 1) * 2)
    call("hps_scheff_field", nr, nz, dptr(np.ascontiguousarray(bins)), dptr(np.ascontiguousarray(mesh)), dptr(out))
    return out


def _noalloc(nr, nz, bins, mesh):
    import torch
    from hpsim_gb300._capi import call, dptr
    b = torch.tensor(bins, dtype=torch.float64, device="cuda")
    # output starts as garbage: the entry point must clear what it sums into
    f = torch.full(((nz + 1) * (nr + 1) * 2,), 7.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    call("hps_scheff_field_noalloc", nr, nz, b.data_ptr(), dptr(np.ascontiguousarray(mesh)), f.data_ptr(),
         stream.cuda_stream)
    stream.synchronize()
    return f.cpu().numpy()


def _case(seed, nr, nz):
    rng = np.random.default_rng(seed)
    bins = rng.uniform(0.0, 4.0, nr * nz) * (rng.uniform(size=nr * nz) > 0.25)
    mesh = np.array([3.5e-4 * (1 + 0.1 * seed), 1.8e-4, 0.045, 201.25, 65536.0, 1.6e-5, float(seed % 2)])
    return bins, mesh


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry_point_on_consecutive_calls():
    from hpsim_gb300 import build
    build.build()
    for seed, (nr, nz) in ((1, (32, 128)), (2, (32, 128)), (3, (16, 64))):
        bins, mesh = _case(seed, nr, nz)
        want = _allocating(nr, nz, bins, mesh)
        got = _noalloc(nr, nz, bins, mesh)
        assert np.allclose(got, want, rtol=1e-9, atol=1e-12 * np.abs(want).max()), (seed, nr, nz)


@pytest.mark.gpu
def test_noalloc_rejects_meshes_beyond_the_static_scratch():
    import ctypes as C
    import torch
    from hpsim_gb300._capi import lib
    b = torch.zeros(64 * 128, dtype=torch.float64, device="cuda")
    f = torch.zeros(129 * 65 * 2, dtype=torch.float64, device="cuda")
    mesh = np.zeros(7)
    st = lib().hps_scheff_field_noalloc(64, 128, b.data_ptr(), mesh.ctypes.data_as(C.POINTER(C.c_double)),
                                        f.data_ptr(), None)
    assert st == HPS_ERR_INVALID
    assert b"too large" in lib().hps_last_error()


def test_noalloc_source_allocates_nothing():
    """The entry point and the launcher it calls contain no allocation."""
    src = open(os.path.join(ROOT, "hpsim_gb300", "csrc", "scheff.cu")).read()
    start = src.index("hps_status hps_scheff_field_noalloc(")
    body = src[start:src.index("}  // extern \"C\"", start)]
    solve = src[src.index("cudaError_t sc_field_solve("):src.index("}  // namespace hps",
                                                                  src.index("cudaError_t sc_field_solve("))]
    for text in (body, solve):
        assert not re.search(r"cudaMalloc|cudaFree|\bmalloc\(|\bnew\b|torch", text)
