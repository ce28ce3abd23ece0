"""Generate the golden fixtures in this directory from the reference's own code.

Runs the reference's tracking code compiled for the host CPU
(oracle/_ref/libhpsref.so, built by `make -C oracle ref` from the reference
tree) on small seeded cases and stores, per case, the lattice records, the
beam set-up, the per-element monitor records and the final particle state.
The fixtures are what the oracle and the CUDA path are checked against where
the reference tree is absent.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from hpsim_gb300 import lattices as L  # noqa: E402
from oracle import refimpl as R  # noqa: E402


def loss_mix():
    """Apertures of both kinds, steerer, rotation, space-charge compensation,
    diagnostics and aperture-limited drift/quad/buncher: a lattice that loses
    particles in several ways."""
    E = L.element
    return [
        E(L.BUNCHER, "B1", voltage=0.12, frequency=201.25, phase=math.radians(-90), aperture=0.0042),
        E(L.DRIFT, "D1", length=0.10, aperture=0.0036),
        E(L.QUAD, "Q1", length=0.05, gradient=18.0, aperture=0.0032),
        E(L.STEERER, "S1", blh=1.0e-4, blv=6.0e-5),
        E(L.APERTURE_C, "AC1", aperture=0.0027),
        E(L.DRIFT, "D2", length=0.10, aperture=0.0031),
        E(L.ROTATION, "R1", angle=0.3),
        E(L.QUAD, "Q2", length=0.05, gradient=-18.0, aperture=0.0029),
        E(L.APERTURE_R, "AR1", xl=0.0021, xr=0.0026, yt=0.0020, yb=0.0023),
        E(L.SPCHCOMP, "SC1", fraction=0.5),
        E(L.DRIFT, "D3", length=0.10),
        E(L.DIAGNOSTICS, "DG1"),
        E(L.QUAD, "Q3", length=0.05, gradient=18.0, aperture=0.0030),
        E(L.DRIFT, "D4", length=0.06, aperture=0.0028),
    ]


def dipole_line():
    E = L.element
    return [
        E(L.QUAD, "Q1", length=0.05, gradient=18.0),
        E(L.DRIFT, "D1", length=0.05),
        E(L.DIPOLE, "BEND1", radius=1.0, angle=0.2, edge_in=0.05, edge_out=0.04, half_gap=0.01,
          k1=0.5, k2=2.8, field_index=0.3, kinetic_energy=0.75),
        E(L.DRIFT, "D2", length=0.05),
        E(L.QUAD, "Q2", length=0.05, gradient=-18.0),
    ]


CASES = {
    # name: (lattice builder, N, space charge or None)
    "fodo_nosc": (lambda: L.small_fodo(), 512, None),
    "fodo_sc": (lambda: L.small_fodo(), 1024, dict(nr=32, nz=128, interval=0.10, remesh_threshold=0.0)),
    "fodo_sc_remesh": (lambda: L.small_fodo(), 1000, dict(nr=32, nz=128, interval=0.05)),
    "dtl_sc": (lambda: L.dtl_like(n_gaps=12), 1024, dict(nr=32, nz=128, remesh_threshold=0.0)),
    "ccl_sc": (lambda: L.ccl_like(modules=1, tanks=2, cells=4), 512, dict(nr=16, nz=64, remesh_threshold=0.0)),
    "loss_mix_sc": (loss_mix, 1024, dict(nr=16, nz=32, interval=0.05, remesh_threshold=0.01)),
    "adj_mesh_cut": (lambda: L.dtl_like(n_gaps=6), 768,
                     dict(nr=16, nz=64, adj_bunch=2, adj_bunch_cutoff_w=0.95, mesh_size_cutoff_w=0.9,
                          remesh_threshold=0.0)),
    "dipole_sc": (dipole_line, 512, dict(nr=16, nz=32, interval=0.02, remesh_threshold=0.0)),
    "tiny_n5": (lambda: L.small_fodo()[:5], 5, dict(nr=8, nz=16, interval=0.1, remesh_threshold=0.0)),
    "tiny_n2": (lambda: L.small_fodo()[:4], 2, dict(nr=8, nz=16, interval=0.1, remesh_threshold=0.0)),
}
SEED = 12345


def make_case(name):
    build, n, spch = CASES[name]
    elems = build()
    types, params, names = L.lattice_arrays(elems)
    twiss = L.waterbag_twiss()
    mon, out = R.run(elems, n, spch=spch, seed=SEED, twiss=twiss)
    meta = dict(name=name, n=n, seed=SEED, twiss=list(twiss), w0=0.75, phi0=0.0, freq=201.25,
                mass=939.294, charge=-1.0, current=0.015, spch=spch, names=names)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), types=types, params=params, mon=mon,
                        meta=json.dumps(meta), **out)
    return mon


def make_waterbag():
    """Initial waterbag and DC distributions (pins the rand() sequence and the
    generators of src/beam/src/beam.cpp:391-537)."""
    lb = R.lib()
    twiss = np.array(L.waterbag_twiss())
    res = {}
    n = 300
    for kind in ("waterbag", "dc"):
        b = lb.ref_beam_create(n, 939.294, -1.0, 0.015)
        if kind == "waterbag":
            lb.ref_beam_set_waterbag(b, R._dp(twiss), 0.1, 0.75, 201.25, 777)
        else:
            lb.ref_beam_set_dc(b, *DC_ARGS)
        out = {k: np.zeros(n) for k in ("x", "xp", "y", "yp", "phi", "w")}
        lo, ll = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
        lb.ref_beam_get(b, *[R._dp(out[k]) for k in ("x", "xp", "y", "yp", "phi", "w")], R._up(lo), R._up(ll))
        lb.ref_beam_free(b)
        for k, v in out.items():
            res[f"{kind}_{k}"] = v
    np.savez_compressed(os.path.join(HERE, "initial_distributions.npz"), twiss=twiss,
                        dc_args=np.array(DC_ARGS, dtype=np.float64), **res)


DC_ARGS = (0.1, 20.0, 3e-3, -0.2, 25.0, 2.5e-3, math.pi, 0.2, 0.75, 4242)


def make_tables():
    """SCHEFF tables after one full solve on an 8x64 mesh (dump layouts of
    src/simulation/src/space_charge.cu:246-304): bins, Green's table,
    field table."""
    elems = [L.element(L.DRIFT, "D1", length=0.02)]
    spch = dict(nr=8, nz=64, interval=0.02, remesh_threshold=0.0)
    nr, nz = 8, 64
    bin_ = np.zeros(nr * nz)
    fld1 = np.zeros((nr + 1) * nr * nz * 2)
    fld2 = np.zeros((nz + 1) * (nr + 1) * 2)
    lb = R.lib()
    b = lb.ref_beam_create(2048, 939.294, -1.0, 0.015)
    tw = np.array(L.waterbag_twiss())
    lb.ref_beam_set_waterbag(b, R._dp(tw), 0.0, 0.75, 201.25, 99)
    lb.ref_beam_set_ref_w(b, 0.75)
    lb.ref_beam_set_ref_phi(b, 0.0)
    bl = lb.ref_beamline_create()
    pp = np.ascontiguousarray(elems[0][2])
    lb.ref_beamline_add(bl, L.DRIFT, b"D1", R._dp(pp))
    sp = lb.ref_scheff_create(nr, nz, 0, 0.02, 0.0, 0.0, 0.0)
    sim = lb.ref_sim_create(b, bl, sp)
    m = np.zeros((1, 24))
    lb.ref_sim_simulate(sim, b, -1, -1, R._dp(m))
    lb.ref_scheff_tables(R._dp(bin_), R._dp(fld1), R._dp(fld2))
    mesh = np.zeros(7)
    lb.ref_scheff_mesh_params(R._dp(mesh))
    np.savez_compressed(os.path.join(HERE, "scheff_tables_8x64.npz"), bin=bin_, fld1=fld1, fld2=fld2, mesh=mesh,
                        mon=m, spch=json.dumps(spch))
    lb.ref_sim_free(sim)
    lb.ref_scheff_free(sp)
    lb.ref_beamline_free(bl)
    lb.ref_beam_free(b)


if __name__ == "__main__":
    if not R.available():
        sys.exit("oracle/_ref/libhpsref.so is missing: run `make -C oracle ref` where the reference tree exists")
    for name in CASES:
        make_case(name)
        print("wrote", name)
    make_waterbag()
    make_tables()
    print("wrote initial_distributions, scheff_tables_8x64")
