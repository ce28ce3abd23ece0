"""Run a lattice through the CUDA path (hpsim_gb300.HPSim over the C ABI)."""
from __future__ import annotations

COORDS = ("x", "xp", "y", "yp", "phi", "w")


def run_gpu(elems, n, spch=None, seed=12345, twiss=None, w0=0.75, phi0=0.0, freq=201.25,
            precision="fp64", monitor=True, graph=True, mass=939.294, charge=-1.0, current=0.015):
    """Waterbag beam through ``elems``; returns (monitor, coords, objects)."""
    from hpsim_gb300 import HPSim, lattices as L
    beam = HPSim.Beam(mass=mass, charge=charge, current=current, num=n, precision=precision)
    beam.set_waterbag(*(twiss or L.waterbag_twiss()), phi0, w0, freq, seed)
    beam.set_ref_w(w0)
    beam.set_ref_phi(phi0)
    bl = HPSim.BeamLine(elements=elems)
    sc = None
    if spch is not None:
        sc = HPSim.SpaceCharge(spch["nr"], spch["nz"], spch.get("interval", 0.01), spch.get("adj_bunch", 0))
        if "remesh_threshold" in spch:
            sc.set_remesh_threshold(spch["remesh_threshold"])
        if "adj_bunch_cutoff_w" in spch:
            sc.set_adj_bunch_cutoff_w(spch["adj_bunch_cutoff_w"])
        if "mesh_size_cutoff_w" in spch:
            sc.set_mesh_size_cutoff_w(spch["mesh_size_cutoff_w"])
    sim = HPSim.Simulator(beam, bl, sc)
    sim.use_graph(graph)
    if monitor:
        sim.enable_monitor(True)
    sim.simulate()
    coords = {k: beam._coord(k) for k in COORDS}
    coords["loss"] = beam._loss(0)
    coords["lloss"] = beam._loss(1)
    mon = sim.monitor.copy() if monitor else None
    return mon, coords, (beam, bl, sc, sim)
