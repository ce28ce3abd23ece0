"""Beam text files: Beam::PrintToFile / Beam::InitBeamFromFile
(src/beam/src/beam.cpp:670-707 and 179-298).

Format: header lines "Info <msg>", "Charge <q>", "Mass <m>", "Current <I>",
"Frequency <f>", then one particle per line with x xp y yp phi w [loss
[lloss]] at 15 significant digits.  The first particle is the reference
particle.
"""
from __future__ import annotations

import re

import numpy as np

_NUM = re.compile(r"^[\s0-9eE+\-.]+$")


def _first_number(line):
    m = re.search(r"[-+]?\d+(\.\d*)?([eE][-+]?\d+)?", line)
    return float(m.group(0)) if m else None


def write_beam_file(path, msg, charge, mass, current, freq, cols, loss, lloss):
    x, xp, y, yp, phi, w = cols
    with open(path, "w") as f:
        f.write(f"Info {msg}\n")
        f.write(f"Charge  {charge:g}\n")
        f.write(f"Mass {mass:g}\n")
        f.write(f"Current {current:g}\n")
        f.write(f"Frequency {freq:g}\n")
        for i in range(len(x)):
            f.write(f"{x[i]:.15g}  {xp[i]:.15g}  {y[i]:.15g}  {yp[i]:.15g}  {phi[i]:.15g}  "
                    f"{w[i]:.15g}  {int(loss[i])}  {int(lloss[i])}\n")


def read_beam_file(path):
    """Return (mass, charge, current, freq, [x, xp, y, yp, phi, w, loss, lloss])."""
    vals = {}
    rows = []
    with open(path) as f:
        for line in f:
            low = line.lower()
            for key in ("charge", "mass", "current", "frequency"):
                if key in low and re.search(r"\d", line):
                    vals[key] = _first_number(line)
            if line.strip() and _NUM.match(line):
                rows.append([float(v) for v in line.split()])
    for key in ("charge", "mass", "current", "frequency"):
        if key not in vals:
            raise ValueError(f"Beam input file error: must define {key} value!")
    ncol = max((len(r) for r in rows), default=6)
    n = len(rows)
    a = np.zeros((n, max(ncol, 8)))
    for i, r in enumerate(rows):
        a[i, :len(r)] = r
    x, xp, y, yp, phi, w = (a[:, k].copy() for k in range(6))
    x[0] = xp[0] = y[0] = yp[0] = 0.0
    loss = a[:, 6].astype(np.uint32) if ncol > 6 else None
    lloss = a[:, 7].astype(np.uint32) if ncol > 7 else None
    return vals["mass"], vals["charge"], vals["current"], vals["frequency"], [x, xp, y, yp, phi, w, loss, lloss]
