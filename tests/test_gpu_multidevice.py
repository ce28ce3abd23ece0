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


def test_objects_refuse_calls_from_another_device():
    """A beam, solver, simulator or batch runs on the device it was made on:
    while another device is current its calls return HPS_ERR_STATE (no
    kernel touches another device's memory), and a simulator cannot join a
    beam and a solver of different devices."""
    import torch
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two visible GPUs")
    from hpsim_gb300 import HPSim, lattices as L
    from hpsim_gb300._capi import dptr, lib
    HPSim.set_gpu(0)
    beam = HPSim.Beam(mass=939.294, charge=-1.0, current=0.015, num=4096, precision="fp32")
    beam.set_waterbag(*L.waterbag_twiss(), 0.0, 0.75, 201.25, 7)
    beam.set_ref_w(0.75)
    sc0 = HPSim.SpaceCharge(32, 128, 0.10, 0)
    sim = HPSim.Simulator(beam, HPSim.BeamLine(elements=L.small_fodo()[:5]), sc0)
    try:
        HPSim.set_gpu(1)
        out = np.zeros(4096)
        assert lib().hps_beam_get_coord(beam.handle, 0, dptr(out)) == 5  # HPS_ERR_STATE
        assert b"device 0" in lib().hps_last_error()
        with pytest.raises(Exception):
            sim.simulate()
        sc1 = HPSim.SpaceCharge(32, 128, 0.10, 0)  # made on device 1
        HPSim.set_gpu(0)
        with pytest.raises(Exception):
            HPSim.Simulator(beam, HPSim.BeamLine(elements=L.small_fodo()[:5]), sc1)
        sim.simulate()  # back on its own device
        assert beam.get_loss_num() == 0
    finally:
        HPSim.set_gpu(0)
