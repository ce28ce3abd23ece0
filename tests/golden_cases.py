"""Load the golden fixtures of tests/golden/ and rerun their set-up."""
from __future__ import annotations

import glob
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
COORDS = ("x", "xp", "y", "yp", "phi", "w")
# monitor columns compared with a relative tolerance (see include/hps_layout.h);
# SC_REMESH (21) is not recorded by the reference driver.
MON_COLS = [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 22]


def case_names():
    """Tracking cases (fixtures with a run description); distributions,
    SCHEFF tables, beam files and lattice records have their own tests."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(p).startswith(("initial_", "scheff_tables", "beam_files", "db_")))


def load(name):
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"), allow_pickle=False)
    meta = json.loads(str(z["meta"]))
    return z, meta


def elems_of(z, meta):
    return [(int(t), n, np.array(p)) for t, n, p in zip(z["types"], meta["names"], z["params"])]


def spch_args(meta):
    s = meta["spch"]
    if s is None:
        return None, None
    args = (s["nr"], s["nz"], s.get("interval", 0.01), s.get("adj_bunch", 0))
    extra = {k: s[k] for k in ("remesh_threshold", "adj_bunch_cutoff_w", "mesh_size_cutoff_w") if k in s}
    return args, extra


def close_rel(a, b, tol, floor=1e-300):
    a, b = np.asarray(a), np.asarray(b)
    scale = np.maximum(np.maximum(np.abs(a), np.abs(b)), floor)
    return np.abs(a - b) / scale <= tol


def monitor_close(m_test, m_ref, rtol, emit_floor=1e-6):
    """Element-wise agreement of two monitor arrays (full HPS_NMON columns).

    Emittances are differences of products; near zero (two particles, a
    collapsed plane) they carry cancellation noise, so they are compared with
    an absolute floor of emit_floor * sigma * sigma'.  NaN agrees with NaN."""
    a, b = np.asarray(m_test, float), np.asarray(m_ref, float)
    ok = close_rel(a, b, rtol) | (np.abs(a - b) < 1e-14) | (np.isnan(a) & np.isnan(b))
    for e, s1, s2 in ((6, 3, 5), (11, 8, 10), (16, 13, 15)):
        scale = np.abs(b[:, s1] * b[:, s2])
        ok[:, e] |= np.abs(np.nan_to_num(a[:, e], nan=0.0) - np.nan_to_num(b[:, e], nan=0.0)) <= emit_floor * scale + 1e-30
    return ok[:, MON_COLS]
