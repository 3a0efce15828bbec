"""The constant tables of the element build's double-float beta(Pe) (VF
variant, csrc/element.cu df_beta_vf), read from the source as text and
checked against their exact values (CPU, no device needed):

* COTH_SERIES[n] = 2^(2n+2) B_(2n+2) / (2n+2)!, the Taylor coefficients of
  coth x - 1/x (Bernoulli numbers), as (hi, lo) FP32 pairs;
* EXP_TAYLOR[n] = 1/n!;
* the three-part ln 2 of the argument reduction (the first part 16
  significant bits, so that k ln2_1 is exact for k < 2^8) and 1/ln 2.

A pair must reproduce its value to 2^-48 relative (the double-float
format's precision)."""
import math
import os
import re
import struct
from fractions import Fraction

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(os.path.dirname(HERE), "vanadis_solver-directional_residual_gb300",
                   "csrc", "element.cu")

# Bernoulli numbers B_2 .. B_20
BERNOULLI = [Fraction(1, 6), Fraction(-1, 30), Fraction(1, 42), Fraction(-1, 30),
             Fraction(5, 66), Fraction(-691, 2730), Fraction(7, 6),
             Fraction(-3617, 510), Fraction(43867, 798), Fraction(-174611, 330)]


def table(name):
    text = open(SRC).read()
    m = re.search(name + r"\[\d+\]\[2\]\s*=\s*\{(.*?)\};", text, re.S)
    assert m, name
    vals = re.findall(r"\{\s*([-0-9a-fx.p+]+)f\s*,\s*([-0-9a-fx.p+]+)f\s*\}", m.group(1))
    return [(Fraction(literal(h)), Fraction(literal(l))) for h, l in vals]


def literal(tok):
    """A C float literal: hexadecimal (0x1.8p-2) or decimal (0.5)."""
    return float.fromhex(tok) if "x" in tok else float(tok)


def assert_pair(pair, exact):
    hi, lo = pair
    # both parts are FP32 values
    for part in (hi, lo):
        f = float(part)
        assert struct.unpack("<f", struct.pack("<f", f))[0] == f, f
    err = abs((hi + lo) - exact)
    assert err <= abs(exact) * Fraction(1, 2 ** 48), (float(exact), float(err / abs(exact)))


def test_coth_series_coefficients():
    rows = table("COTH_SERIES")
    assert len(rows) == 10
    for n, pair in enumerate(rows, start=1):
        exact = Fraction(2 ** (2 * n)) * BERNOULLI[n - 1] / math.factorial(2 * n)
        assert_pair(pair, exact)


def test_exp_taylor_coefficients():
    rows = table("EXP_TAYLOR")
    assert len(rows) == 8
    for n, pair in enumerate(rows):
        assert_pair(pair, Fraction(1, math.factorial(n)))


def test_ln2_reduction_constants():
    text = open(SRC).read()
    body = text[text.index("__device__ __forceinline__ Df2 df_beta_vf"):]
    body = body[:body.index("\n}\n")]
    consts = list(dict.fromkeys(re.findall(r"(0x1\.[0-9a-f]+p[-+]?\d+)f", body)))
    inv_ln2, l1, l2, l3 = (float.fromhex(c) for c in consts[:4])
    ln2 = Fraction("0.69314718055994530941723212145817656807550013436025525412")
    assert abs(inv_ln2 - 1 / float(ln2)) <= 2 ** -24
    # ln2_1 has at most 16 significant bits: k ln2_1 is exact for k < 2^8
    m1 = Fraction(l1) * 2 ** 16
    assert m1.denominator == 1 and m1 < 2 ** 16
    total = Fraction(l1) + Fraction(l2) + Fraction(l3)
    assert abs(total - ln2) < Fraction(1, 2 ** 68)
