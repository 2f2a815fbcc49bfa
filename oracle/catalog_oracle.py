"""CPU oracle of the catalog reader (test infrastructure: only the tests
import it).  Restates the reading rules CSV.jl applies in the reference's
examples (``examples/lightcone.jl:22-23``: whitespace-delimited FP32
columns) with an exact decimal-to-FP32 conversion: the token is read as an
exact rational and rounded to the nearest FP32, ties to even."""
from __future__ import annotations

import math
import struct
from fractions import Fraction

import numpy as np


def _f32_bits_to_float(b):
    return struct.unpack("<f", struct.pack("<I", b))[0]


def _exact_fraction_of_f32(v):
    return Fraction(float(v))     # FP32 values are exact in FP64


def to_f32(token: str) -> np.float32:
    """Correctly rounded FP32 of a decimal token (no inf/nan handling beyond
    overflow to inf)."""
    q = Fraction(token.strip())     # exact rational of the decimal text
    if q == 0:
        return np.float32(-0.0) if token.strip().startswith("-") else np.float32(0.0)
    sign = -1 if q < 0 else 1
    a = abs(q)
    # candidate from FP64 (within one FP32 ulp), then exact neighbour test
    with np.errstate(over="ignore"):
        c = np.float32(float(a))
        if not np.isfinite(c):
            c = np.float32(np.finfo(np.float32).max)
    lo, hi = c, c
    if Fraction(float(c)) > a:
        lo = np.nextafter(c, np.float32(0))
    else:
        with np.errstate(over="ignore"):
            hi = np.nextafter(c, np.float32(np.inf))
    if not np.isfinite(hi):
        mid_hi = Fraction(float(lo)) + Fraction(2) ** (127 - 23) / 2   # half an ulp above FLT_MAX
        return np.float32(sign * (np.inf if a >= mid_hi else float(lo)))
    flo, fhi = Fraction(float(lo)), Fraction(float(hi))
    mid = (flo + fhi) / 2
    if a < mid:
        r = lo
    elif a > mid:
        r = hi
    else:
        bits_lo = struct.unpack("<I", struct.pack("<f", float(lo)))[0]
        r = lo if bits_lo % 2 == 0 else hi
    return np.float32(sign * float(r))


def read_ascii(text: str, usecols, skip=0, comment="#"):
    """Columns of a whitespace-delimited catalog given as text."""
    rows = []
    for i, line in enumerate(text.split("\n")):
        if i < skip:
            continue
        s = line.strip()
        if not s or (comment and s.startswith(comment)):
            continue
        f = s.split()
        if len(f) <= max(usecols):
            raise ValueError(f"line {i + 1}: too few fields")
        rows.append([to_f32(f[c]) for c in usecols])
    return [np.array([r[k] for r in rows], np.float32) for k in range(len(usecols))]
