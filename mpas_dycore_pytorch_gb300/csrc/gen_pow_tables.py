"""Writes pow_tables.inc, the tables of pow_exner.cuh, from exact decimal arithmetic.

* log table, j = 0..255: c_j = 1 + (j + 1/2) / 256 (exact in binary); 1/c_j and ln(c_j),
  each as an unevaluated sum hi + lo of two doubles (hi = the double nearest the value,
  lo = the double nearest the remainder);
* exp table, j = 0..255: 2**(j / 256) as hi + lo;
* split constants: ln 2 = LN2_HI + LN2_LO with LN2_HI on 42 significant bits (so that
  e * LN2_HI is exact for every binary exponent e), ln(2) / 256 = L256_HI + L256_LO with
  L256_HI on 34 bits (k * L256_HI exact for |k| < 2**19), 256 / ln 2;
* Taylor coefficients (-1)**(n+1) / n (n = 3..10) of log1p and 1 / n! (n = 3..7) of exp.

Every double is the correctly rounded value of a 60-digit decimal (Python's decimal
module rounds ln, exp and power correctly at its context precision).

Run:  python mpas_dycore_pytorch_gb300/csrc/gen_pow_tables.py  (rewrites pow_tables.inc)
"""

from __future__ import annotations

import math
import pathlib
import sys
from decimal import Decimal, getcontext
from fractions import Fraction

getcontext().prec = 60
HERE = pathlib.Path(__file__).resolve().parent


def hi_lo(d: Decimal) -> tuple[float, float]:
    hi = float(d)
    return hi, float(d - Decimal(hi))


def split_bits(d: Decimal, bits: int) -> tuple[float, float]:
    e = math.frexp(float(d))[1]
    hi = math.ldexp(math.floor(math.ldexp(float(d), bits - e)), e - bits)
    return hi, float(d - Decimal(hi))


def render() -> str:
    ln2 = Decimal(2).ln()
    lines = ["// Generated by gen_pow_tables.py from 60-digit decimal arithmetic; do not edit.",
             "// {1/c hi, 1/c lo, ln c hi, ln c lo} for c = 1 + (j + 1/2) / 256"]
    lines.append("MPASG_POW_TABLE double kPowLogTab[256][4] = {")
    for j in range(256):
        c = Decimal(1) + (Decimal(j) + Decimal("0.5")) / 256
        ih, il = hi_lo(1 / c)
        lh, ll = hi_lo(c.ln())
        lines.append(f"  {{{ih!r}, {il!r}, {lh!r}, {ll!r}}},")
    lines.append("};")
    lines.append("// {2^(j/256) hi, lo}")
    lines.append("MPASG_POW_TABLE double kPowExpTab[256][2] = {")
    for j in range(256):
        th, tl = hi_lo(Decimal(2) ** (Decimal(j) / 256))
        lines.append(f"  {{{th!r}, {tl!r}}},")
    lines.append("};")
    l2h, l2l = split_bits(ln2, 42)
    lkh, lkl = split_bits(ln2 / 256, 34)
    lines.append(f"constexpr double kPowLn2Hi = {l2h!r};")
    lines.append(f"constexpr double kPowLn2Lo = {l2l!r};")
    lines.append(f"constexpr double kPowL256Hi = {lkh!r};")
    lines.append(f"constexpr double kPowL256Lo = {lkl!r};")
    lines.append(f"constexpr double kPowInvL256 = {float(256 / ln2)!r};")
    for n in range(3, 11):
        lines.append(f"constexpr double kPowLogC{n} = {float(Fraction((-1) ** (n + 1), n))!r};")
    for n in range(3, 8):
        lines.append(f"constexpr double kPowExpC{n} = {float(Fraction(1, math.factorial(n)))!r};")
    return "\n".join(lines) + "\n"


if __name__ == "__main__":
    text = render()
    if len(sys.argv) > 1 and sys.argv[1] == "--check":
        sys.exit(0 if (HERE / "pow_tables.inc").read_text() == text else 1)
    (HERE / "pow_tables.inc").write_text(text)
