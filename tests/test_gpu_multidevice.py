"""Kernel attributes are per device: the large dynamic shared-memory limits of
the deposit, contraction and network kernels are set on every device the
process uses, not only on the first.  One process switches devices and runs
the FP32 and FP64 space-charge paths and the field solves on each; with
fewer than two GPUs visible the test is skipped."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fp32_run(device):
    from hpsim_gb300 import HPSim, lattices as L
    HPSim.set_gpu(device)
    beam = HPSim.Beam(mass=939.294, charge=-1.0, current=0.015, num=8192, precision="fp32")
    beam.set_waterbag(*L.waterbag_twiss(), 0.0, 0.75, 201.25, 99)
    beam.set_ref_w(0.75)
    sc = HPSim.SpaceCharge(32, 128, 0.10, 0)
    sim = HPSim.Simulator(beam, HPSim.BeamLine(elements=L.small_fodo()[:7]), sc)
    sim.enable_monitor(True)
    sim.simulate()
    return sim.monitor.copy()


def test_switching_devices_in_one_process():
    import torch
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two visible GPUs")
    from hpsim_gb300 import HPSim
    from hpsim_gb300._capi import call, dptr
    mons = [_fp32_run(d) for d in (0, 1)]
    assert np.array_equal(mons[0], mons[1])
    nr, nz = 32, 128
    rng = np.random.default_rng(5)
    bins = rng.uniform(0.0, 4.0, nr * nz)
    mesh = np.array([3.5e-4, 1.8e-4, 0.045, 201.25, 65536.0, 1.6e-5, 0.0])
    fields = []
    for d in (0, 1):
        HPSim.set_gpu(d)
        torch.cuda.set_device(d)
        b = torch.tensor(bins, dtype=torch.float64, device=f"cuda:{d}")
        f = torch.zeros((nz + 1) * (nr + 1) * 2, dtype=torch.float64, device=f"cuda:{d}")
        s = torch.cuda.current_stream(d)
        call("hps_scheff_field_noalloc", nr, nz, b.data_ptr(), dptr(mesh), f.data_ptr(), s.cuda_stream)
        s.synchronize()
        fields.append(f.cpu().numpy())
    assert np.array_equal(fields[0], fields[1])
    HPSim.set_gpu(0)
    torch.cuda.set_device(0)
