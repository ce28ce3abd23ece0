"""Element records of two of the reference's lattice databases, for GPU
parity runs on real lattices where the databases are not available.

    python tests/golden/make_db_lattices.py [db_dir]

Reads (read-only) ``dtl.db`` (the LANSCE DTL: 165 gaps, 170 quads, 0.75 ->
99.5 MeV) and ``tbtd.db`` (a 0.75 MeV transport line with dipoles,
bunchers, steerers, rectangular and circular apertures and space-charge
compensation) through hpsim_gb300.dbloader and stores types, names and the
32-slot parameter records with the beam settings the parity tests use.  The
input phase of the DTL beam (-2.7 rad) is inside the range the oracle
transmits fully with space charge; the transport line loses most of this
synthetic beam on its apertures, which the tests use as loss-flag cases.
"""
import os
import sqlite3
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from hpsim_gb300 import dbloader  # noqa: E402

RUNS = {
    "dtl": dict(w0=0.75, phi0=-2.7, freq=201.25),
    "tbtd": dict(w0=0.75, phi0=0.0, freq=201.25),
}


class _Conn:
    def __init__(self, path):
        self._conn = sqlite3.connect(f"file:{path}?mode=ro", uri=True)
        self.dbs = [("main", path)]
        self.model_index = {}


def load(db_dir, name):
    return dbloader.generate_beamline(_Conn(os.path.join(db_dir, f"{name}.db")))


def main(db_dir):
    for name, run in RUNS.items():
        els = load(db_dir, name)
        np.savez_compressed(os.path.join(HERE, f"db_{name}.npz"),
                            types=np.array([e[0] for e in els], dtype=np.int32),
                            names=np.array([e[1] for e in els]),
                            params=np.stack([e[2] for e in els]),
                            **{k: np.float64(v) for k, v in run.items()})
        print(name, len(els), "elements")


if __name__ == "__main__":
    # the reference's databases: the argument, else $HPS_REFERENCE_DB, else
    # the "reference" checkout beside this repository
    default = os.environ.get("HPS_REFERENCE_DB", os.path.join(HERE, "..", "..", "..", "reference", "db"))
    main(sys.argv[1] if len(sys.argv) > 1 else default)
