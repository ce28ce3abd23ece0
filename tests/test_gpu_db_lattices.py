"""Real lattices from the reference's databases (fixtures made by
tests/golden/make_db_lattices.py through hpsim_gb300/dbloader.py): the
LANSCE DTL (349 elements, 0.75 -> 99.5 MeV) and the 0.75 MeV transport
line (dipoles, bunchers, steerers, apertures, space-charge compensation),
with SCHEFF 32 x 128, through the CUDA path against the FP64 oracle.

FP64: loss flags exact, statistics within 1e-6 relative.  FP32: loss flags
exact, statistics within the FP32 path's stated tolerances."""
import os

import numpy as np
import pytest

from tests import golden_cases as G
from tests.gpu_runs import run_gpu
from tests.test_gpu_fp32 import assert_fp32_close

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
N = 16384


def lattice(name):
    z = np.load(os.path.join(HERE, "golden", f"db_{name}.npz"))
    elems = [(int(t), str(n), p) for t, n, p in zip(z["types"], z["names"], z["params"])]
    return elems, {k: float(z[k]) for k in ("w0", "phi0", "freq")}


@pytest.fixture(scope="module")
def oracle_runs(oracle):
    out = {}
    for name in ("dtl", "tbtd"):
        elems, run = lattice(name)
        out[name] = oracle.run(elems, N, spch_args=(32, 128, 0.01, 0), **run)
    return out


@pytest.mark.parametrize("name", ["dtl", "tbtd"])
def test_db_lattice_fp64_matches_oracle(name, oracle_runs):
    elems, run = lattice(name)
    mon, c, _ = run_gpu(elems, N, spch=dict(nr=32, nz=128), **run)
    mo, co = oracle_runs[name]
    assert np.array_equal(c["loss"], co["loss"]), (name, np.flatnonzero(c["loss"] != co["loss"])[:10])
    assert np.array_equal(c["lloss"], co["lloss"]), name
    ok = G.monitor_close(mon, mo, 1e-6)
    assert ok.all(), (name, np.argwhere(~ok)[:5])
    if name == "dtl":  # the beam is accelerated and transmitted
        alive = c["loss"] == 0
        assert alive.mean() > 0.99 and c["w"][alive].mean() > 99.0


@pytest.mark.parametrize("name", ["dtl", "tbtd"])
def test_db_lattice_fp32_matches_oracle(name, oracle_runs):
    elems, run = lattice(name)
    mon, c, _ = run_gpu(elems, N, spch=dict(nr=32, nz=128), precision="fp32", **run)
    mo, co = oracle_runs[name]
    assert np.array_equal(c["loss"], co["loss"]), (name, np.flatnonzero(c["loss"] != co["loss"])[:10])
    assert np.array_equal(c["lloss"], co["lloss"]), name
    assert_fp32_close(mon, mo, name)
