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


def _first_number(line):
    """GetFirstNumberInString (src/util/src/utility.cpp:31-74): digits with
    one optional sign (only directly before a digit) and one dot, stopping at
    the first other character -- no exponent, so '1.5e-05' reads as 1.5."""
    out, started, dot = [], False, False
    for i, ch in enumerate(line):
        if ch in "+-":
            if not started and i < len(line) - 1 and line[i + 1].isdigit():
                started = True
                out.append(ch)
            elif started:
                break
        elif ch == ".":
            if started and not dot:
                out.append(ch)
                dot = True
            elif dot:
                break
        elif ch.isdigit():
            out.append(ch)
            started = True
        elif started:
            break
    return _atof("".join(out))


def _atof(s):
    """std::atof: the longest leading number, 0 when there is none."""
    m = re.match(r"\s*[-+]?(\d+(\.\d*)?|\.\d+)([eE][-+]?\d+)?", s)
    return float(m.group(0)) if m else 0.0


def _atoi(s):
    m = re.match(r"\s*[-+]?\d+", s)
    return int(m.group(0)) if m else 0


def _contains_numbers(line):
    return any(ch.isdigit() for ch in line)


def _only_numbers(line):
    """ContainOnlyNumbers (utility.cpp:98-110): with the spaces removed (only
    spaces), every character is a digit, '.', '-', 'e' or 'E'; a line with a
    tab or a '+' is not a particle line."""
    s = line.rstrip("\n").replace(" ", "")
    return bool(s) and all(ch.isdigit() or ch in ".-eE" for ch in s)


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
    """Beam::InitBeamFromFile + UpdateBeamFromFile (beam.cpp:179-298).

    Returns (mass, charge, current, freq, [x, xp, y, yp, phi, w, loss,
    lloss]).  Header values: the first number of the last line that
    mentions the key (case-insensitive) and holds a digit.  Particle lines:
    those of numbers only; the loss columns are read when the *last*
    particle line has them (a shorter line then gives 0 where the reference
    leaves the value unset).  The first particle is put on axis."""
    vals = {}
    rows = []
    with open(path) as f:
        for line in f:
            low = line.lower()
            for key in ("charge", "mass", "current", "frequency"):
                if key in low and _contains_numbers(line):
                    vals[key] = _first_number(line)
            if _only_numbers(line):
                rows.append(line.split())
    for key in ("charge", "mass", "current", "frequency"):
        if key not in vals:
            raise ValueError(f"Beam input file error: must define {key} value!")
    if not rows:
        raise ValueError("Beam input file error: no particle lines")
    n = len(rows)
    cols = [np.zeros(n) for _ in range(6)]
    loss = np.zeros(n, dtype=np.uint32)
    lloss = np.zeros(n, dtype=np.uint32)
    for i, r in enumerate(rows):
        for k in range(6):
            cols[k][i] = _atof(r[k]) if k < len(r) else 0.0
        if len(r) > 6:
            loss[i] = _atoi(r[6]) & 0xffffffff
        if len(r) > 7:
            lloss[i] = _atoi(r[7]) & 0xffffffff
    ncol = len(rows[-1])
    x, xp, y, yp, phi, w = cols
    x[0] = xp[0] = y[0] = yp[0] = 0.0
    return (vals["mass"], vals["charge"], vals["current"], vals["frequency"],
            [x, xp, y, yp, phi, w, loss if ncol > 6 else None, lloss if ncol > 7 else None])
