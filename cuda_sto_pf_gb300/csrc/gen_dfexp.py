"""Generate dfexp.cuh: constants of the double-float exponential.

    python cuda_sto_pf_gb300/csrc/gen_dfexp.py

A double-float value is an unevaluated sum hi + lo of two floats (about 48
significant bits).  The exponential of a double-float w <= 0 is taken as
    e^w = 2^k * 2^(j/64) * e^r,   w = (64 k + j) ln2/64 + r,  |r| <= ln2/128,
with 2^(j/64) (j = 0..63) from a double-float table and ln2/64 split into
three floats, the first with 12 significant bits so that N * C1 is exact for
|N| < 4096 (|w| <= 40).  All values are computed here in 60-digit decimal
arithmetic and rounded to float by exact rational comparison.
"""
import os
from decimal import Decimal, getcontext
from fractions import Fraction

import numpy as np

getcontext().prec = 60
HERE = os.path.dirname(os.path.abspath(__file__))


def to_f32(x):
    """nearest float to the rational/decimal x (ties: the one numpy picks)"""
    f = Fraction(x)
    c = np.float32(float(f))
    # float(f) is the nearest double; step to the nearest float by comparison
    best = c
    for cand in (np.nextafter(c, np.float32(-np.inf)), c, np.nextafter(c, np.float32(np.inf))):
        if abs(Fraction(float(cand)) - f) < abs(Fraction(float(best)) - f):
            best = cand
    return best


def split(x):
    hi = to_f32(x)
    lo = to_f32(Fraction(x) - Fraction(float(hi)))
    return hi, lo


def flit(v):
    v = float(v)
    return "0.0f" if v == 0.0 else f"{float.hex(v)}f" if False else f"{np.float32(v).item():.9e}f"


def hexf(v):
    # exact float literal: C hexadecimal floating constant
    return float(np.float32(v)).hex() + "f"


def main():
    ln2 = Decimal(2).ln()
    l64 = Fraction(ln2) / 64
    c1 = Fraction(round(l64 * 2**18), 2**18)        # 12 significant bits (ln2/64 ~ 1.39 * 2^-7)
    assert c1.numerator < 4096
    c2 = to_f32(l64 - c1)
    c3 = to_f32(l64 - c1 - Fraction(float(c2)))
    tab = []
    for j in range(64):
        v = Decimal(2) ** (Decimal(j) / Decimal(64))
        tab.append(split(Fraction(v)))
    lines = ["// Generated by gen_dfexp.py -- constants of the double-float exponential.",
             "#pragma once", "",
             "namespace dfexp {",
             f"constexpr float kInvL64 = {hexf(to_f32(1 / l64))};   // 64 / ln2",
             f"constexpr float kC1 = {hexf(float(c1))};   // ln2/64 = C1 + C2 + C3, C1 with 12 bits",
             f"constexpr float kC2 = {hexf(c2)};",
             f"constexpr float kC3 = {hexf(c3)};",
             "// 2^(j/64) = x + y (hi, lo); indexed at run time, so a device array that",
             "// kernels copy to shared memory (a local constexpr table would be",
             "// rebuilt in local memory on every call)",
             "static __device__ const float2 kExp2Tab[64] = {",
             *["    {" + hexf(h) + ", " + hexf(l) + "}," for h, l in tab],
             "};",
             "}  // namespace dfexp", ""]
    with open(os.path.join(HERE, "dfexp.cuh"), "w") as f:
        f.write("\n".join(lines))


if __name__ == "__main__":
    main()
