"""Beam text files written and read by the reference's own Beam class
(Beam::PrintToFile, Beam(file); src/beam/src/beam.cpp:47-60, 179-298,
670-707), compiled for the host from the reference tree by oracle/Makefile
(oracle/_ref/libhpsref.so), for tests/test_beam_io.py.

    make -C oracle ref && python tests/golden/make_beam_files.py

Stores: the text PrintToFile writes for a ten-particle beam with loss flags,
and, for a file with the format's corner cases (an exponent in a header
value, a tab-separated line, a line with a '+' exponent, a message line that
mentions a key), what the reference's reader makes of it.
"""
import ctypes as C
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

QUIRKS = """Info charge of 7 is not the charge
Charge  -1
Mass 939.294
Current 1.5e-02 (read as 1.5: no exponents in header values)
Frequency 201.25 MHz
0  0  0  0  0.1  0.75  0  0
0.001  -0.002  0.0015  2.5e-05  -0.03  0.76  0  0
-0.0004\t0.001\t0.0002\t0.0003\t0.01\t0.74\t0\t0
0.002  0.001  -0.001  0.0004  1e+01  0.75  0  0
0.0003  0.0001  0.0002  -0.0001  0.02  0.751  5  1
-1.25e-03  3.5E-04  0.0001  0.0002  -0.015  0.749  0  1
"""


def lib():
    return C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libhpsref.so"))


def dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def up(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint))


def read_back(L, b):
    n = L.ref_beam_size(b)
    arrs = [np.zeros(n) for _ in range(6)]
    loss, lloss = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
    L.ref_beam_get(b, *[dp(a) for a in arrs], up(loss), up(lloss))
    sc = np.zeros(5)
    L.ref_beam_scalars(b, dp(sc))
    return arrs, loss, lloss, sc


def main():
    L = lib()
    L.ref_beam_create.restype = C.c_void_p
    L.ref_beam_from_file.restype = C.c_void_p
    L.ref_beam_size.restype = C.c_uint
    for f in ("ref_beam_free", "ref_beam_print", "ref_beam_get", "ref_beam_scalars", "ref_beam_size",
              "ref_beam_set_distribution", "ref_beam_set_frequency"):
        getattr(L, f).argtypes = None
    L.ref_beam_free.argtypes = [C.c_void_p]
    L.ref_beam_size.argtypes = [C.c_void_p]
    rng = np.random.default_rng(3)
    n = 10
    cols = [rng.normal(scale=s, size=n) for s in (1e-3, 1e-3, 1e-3, 1e-3, 0.1)] + [0.75 + 1e-3 * rng.normal(size=n)]
    cols[0][3] = 1.2345678901234567e-7
    loss = np.array([0, 0, 12, 0, 33333333, 0, 9999, 0, 0, 99999], dtype=np.uint32)
    lloss = np.array([0, 1, 0, 0, 0, 0, 0, 1, 0, 0], dtype=np.uint32)
    b = C.c_void_p(L.ref_beam_create(C.c_uint(n), C.c_double(939.294), C.c_double(-1.0), C.c_double(0.015)))
    L.ref_beam_set_distribution(b, *[dp(np.ascontiguousarray(c)) for c in cols], up(loss), up(lloss))
    L.ref_beam_set_frequency(b, C.c_double(201.25))
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "print.txt")
        L.ref_beam_print(b, out.encode(), b"golden beam")
        printed = open(out).read()
        L.ref_beam_free(b)
        qf = os.path.join(td, "quirks.txt")
        open(qf, "w").write(QUIRKS)
        rb = C.c_void_p(L.ref_beam_from_file(qf.encode()))
        arrs, rloss, rlloss, sc = read_back(L, rb)
        L.ref_beam_free(rb)
    np.savez(os.path.join(HERE, "beam_files.npz"), print_cols=np.stack(cols), print_loss=loss,
             print_lloss=lloss, print_text=np.array(printed), quirks_text=np.array(QUIRKS),
             quirks_cols=np.stack(arrs), quirks_loss=rloss, quirks_lloss=rlloss, quirks_scalars=sc)
    print(printed[:300])
    print("read", len(arrs[0]), "particles; scalars (mass, charge, current, freq, design_w)", sc)


if __name__ == "__main__":
    sys.exit(main())
