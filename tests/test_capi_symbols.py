"""The C-ABI library builds, loads and exports every entry point that
include/*.h declares (host-only checks; nothing here needs a GPU)."""
import ctypes as C
import os
import re

import pytest

from tests.conftest import ROOT

HEADERS = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")]


def declared_symbols():
    names = set()
    for h in HEADERS:
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:hps_status|int|const char \*|uint64_t)\s*(hps_\w+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def capi():
    from hpsim_gb300 import build
    build.build()
    from hpsim_gb300 import _capi
    return _capi


def test_headers_declare_the_abi():
    syms = declared_symbols()
    assert len(syms) >= 40
    for s in ("hps_beam_create", "hps_sim_simulate", "hps_scheff_create", "hps_beamline_add"):
        assert s in syms


def test_library_exports_every_declared_symbol(capi):
    lib = C.CDLL(capi.library_path())
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_abi_version_and_status_strings(capi):
    L = capi.lib()
    assert L.hps_abi_version() == 1
    assert L.hps_status_string(0) == b"ok"
    assert L.hps_status_string(4) == b"malformed lattice"


def test_beamline_host_side(capi):
    """BeamLine construction and case-insensitive lookup are host-only."""
    import numpy as np
    from hpsim_gb300 import lattices as L
    lib = capi.lib()
    h = C.c_void_p()
    capi.check(lib.hps_beamline_create(C.byref(h)))
    for t, name, p in L.small_fodo()[:5]:
        capi.check(lib.hps_beamline_add(h, t, name.encode(), capi.dptr(np.ascontiguousarray(p))))
    idx = C.c_uint32()
    capi.check(lib.hps_beamline_find(h, b"qm01", C.byref(idx)))
    assert idx.value == 4
    assert lib.hps_beamline_find(h, b"nope", C.byref(idx)) == 3  # HPS_ERR_NOT_FOUND
    assert b"nope" in lib.hps_last_error()
    n = C.c_uint32()
    capi.check(lib.hps_beamline_size(h, C.byref(n)))
    assert n.value == 5
    capi.check(lib.hps_beamline_destroy(h))


def test_invalid_handles_are_rejected(capi):
    lib = capi.lib()
    assert lib.hps_sim_simulate(None, 0, -1) == 1
    assert lib.hps_beam_get_coord(None, 0, None) == 1
    bad = C.c_void_p()
    assert lib.hps_scheff_create(48, 128, 0, C.byref(bad)) == 1  # not a power of two


def test_beam_particle_count_limit(capi):
    """A beam holds at most 2^31 particles (the reference's next-power-of-two
    launch geometry and 32-bit particle indices); the check runs before any
    device work."""
    lib = capi.lib()
    out = C.c_void_p()
    for prec in (0, 1):
        assert lib.hps_beam_create((1 << 31) + 1, 939.294, -1.0, 0.0, prec, C.byref(out)) == 1
        assert not out.value
        assert b"2^31" in lib.hps_last_error()
