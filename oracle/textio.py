"""CPU restatement of the reference's text outputs of a time step.

TEST INFRASTRUCTURE ONLY: the oracle of the library's text writers
(``vdr_write_result_txt``, ``vdr_write_slices_txt``); the product never
imports it.

* ``result_txt`` follows vanadis_full_DR_OpenMP_timing.for:797-806: one line
  per node, ``write(nout10, 122) xx(i), yy(i), zz(i), tnw2(i) * 1d6`` with
  ``122 format (e12.5, 2x, e12.5, 2x, e12.5, 2x, e12.5)``.
* ``split_result_txt`` follows vanadis_files (:1089-1184) step by step: it
  READs the T file back with format 222 and writes the X/Y/Z slice records
  with ``125 format (e12.5, 2x, e12.5, 2x, e12.5)`` and the index formulas
  of its three loops.
* ``fortran_e`` is the Fortran standard's Ew.d output edit (d significant
  digits after "0.", exponent E+ee for |exp| <= 99 and +eee up to 999), its
  digits from Python's correctly rounded float formatting (round to
  nearest, ties to even on exact binary ties).  gfortran's rounding of exact
  decimal ties is processor-dependent; no recorded output of the reference
  pins it, so exact binary ties are a convention of this oracle.
"""
from __future__ import annotations

import math

import numpy as np


def fortran_e(v: float, w: int = 12, d: int = 5) -> str:
    """Ew.d edit of v (w = 12, d = 5 in the reference's formats)."""
    v = float(v)
    if math.isnan(v):
        return "NaN".rjust(w)
    if math.isinf(v):
        return ("-Infinity" if v < 0 else "Infinity").rjust(w)
    s = "%.*e" % (d - 1, v)           # [-]d.dddde(+|-)xx
    neg = s.startswith("-")
    mant, ex = s.lstrip("-").split("e")
    digits = mant.replace(".", "")
    fe = 0 if v == 0.0 else int(ex) + 1
    if abs(fe) <= 99:
        es = "E%s%02d" % ("-" if fe < 0 else "+", abs(fe))
    else:
        es = "%s%03d" % ("-" if fe < 0 else "+", abs(fe))
    out = ("-" if neg else "") + "0." + digits + es
    return out.rjust(w)


def fortran_read_e(field: str) -> float:
    """READ with an Ew.d edit of one field (the forms fortran_e writes)."""
    f = field.strip()
    if f in ("NaN",):
        return float("nan")
    if f.endswith("Infinity"):
        return float("-inf") if f.startswith("-") else float("inf")
    if "E" not in f:  # 0.ddddd+eee: the exponent letter is dropped
        k = max(f.rfind("+"), f.rfind("-"))
        f = f[:k] + "E" + f[k:]
    return float(f)


def result_txt(xx, yy, zz, t, scale: float = 1e6) -> bytes:
    """The text of T_sssss.TXT (format 122)."""
    lines = []
    for x, y, z, v in zip(xx, yy, zz, t):
        lines.append("  ".join(fortran_e(a) for a in (x, y, z, float(v) * scale)))
    return ("\n".join(lines) + ("\n" if lines else "")).encode()


def read_result_txt(text: bytes):
    """READ (9, 222) x1(i), x2(i), x3(i), s(i) for every line."""
    rows = []
    for line in text.decode().splitlines():
        fields = [line[0:12], line[14:26], line[28:40], line[42:54]]
        rows.append([fortran_read_e(f) for f in fields])
    a = np.array(rows, dtype=np.float64).reshape(-1, 4)
    return a[:, 0], a[:, 1], a[:, 2], a[:, 3]


def _rec3(a, b, c) -> str:
    return "  ".join(fortran_e(v) for v in (a, b, c))


def split_result_txt(text: bytes, nx1: int, nx2: int, nx3: int, step: int) -> dict:
    """vanadis_files for one step: {file name: bytes} of the X, Y and Z
    slice files split from the text of T_sssss.TXT."""
    x1, x2, x3, s = read_result_txt(text)
    x, y, z = nx1, nx2, nx3
    out = {}
    for j in range(1, x + 1):            # dane_x(j): x2, x3, s of node x (i-1) + j
        recs = []
        for i in range(1, y * z + 1):
            n = x * (i - 1) + 1 + j - 1 - 1
            recs.append(_rec3(x2[n], x3[n], s[n]))
        out["X_%05d_%03d.TXT" % (step, j)] = ("\n".join(recs) + "\n").encode()
    for j in range(1, y + 1):            # dane_y(j): x3, x1, s, k counts planes
        recs = []
        k = 1
        for i in range(1, x * z + 1):
            if (i - 1) % x == 0 and (i - 1) != 0:
                k += 1
            n = i + x * (j - 1) + x * (y - 1) * (k - 1) - 1
            recs.append(_rec3(x3[n], x1[n], s[n]))
        out["Y_%05d_%03d.TXT" % (step, j)] = ("\n".join(recs) + "\n").encode()
    for j in range(1, z + 1):            # dane_z(j): x2, x1, s of node i + x y (j-1)
        recs = []
        for i in range(1, x * y + 1):
            n = i + x * y * (j - 1) - 1
            recs.append(_rec3(x2[n], x1[n], s[n]))
        out["Z_%05d_%03d.TXT" % (step, j)] = ("\n".join(recs) + "\n").encode()
    return out
