"""GB300 implementation of HPSim's per-element particle-tracking path.

``hpsim_gb300.HPSim`` mirrors the reference's ``HPSim`` extension module
(Beam, BeamLine, SpaceCharge, Simulator, DBConnection, set_gpu) over the C
ABI of include/hpsim_gb300.h; ``hpsim_gb300.lattices`` builds element records
and the synthetic benchmark lattices.
"""
from . import lattices  # noqa: F401
