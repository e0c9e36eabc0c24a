"""Elementary functions built from IEEE 754 basic operations only.

The synthetic cases (``cases.py``) have to come out bit-identical on every machine, so
that a run on the GPU host starts from the very arrays a reference run started from on
another machine: a one-ulp difference in a cell area or an edge length grows to ~1e-10
in the divergence after two large steps.  NumPy's transcendental ufuncs cannot promise
that: they dispatch to platform-specific SIMD or libm code whose last bit differs between
x86-64 and aarch64.  Every function here is built from ``+ - * /`` and ``sqrt`` (correctly
rounded by IEEE 754 everywhere), exact scalings (``ldexp`` / ``frexp``), ``rint`` and
comparisons, each a separate NumPy ufunc (NumPy never fuses them into multiply-adds), and
from constants derived here from decimal expansions with exact rational arithmetic.  The
results are accurate to a few units in the last place; what matters is that they are the
same everywhere.

Methods: Cody-Waite argument reduction with a split constant (exp, sin, cos), the
atanh series of ``(m - 1) / (m + 1)`` (log), two half-angle steps before the arctangent
series (atan), Taylor polynomials evaluated by Horner's rule.
"""

from __future__ import annotations

import math
from decimal import Decimal, getcontext
from fractions import Fraction

import numpy as np

getcontext().prec = 60
_LN2 = Decimal("0.693147180559945309417232121458176568075500134360255254120680009")
_PI = Decimal("3.14159265358979323846264338327950288419716939937510582097494459")


def _split(d: Decimal, bits: int) -> tuple[float, float]:
    """``d`` as hi + lo: hi keeps ``bits`` significant bits (so small integer multiples
    of it are exact), lo is the rest rounded to a double."""
    e = math.frexp(float(d))[1]
    hi = math.ldexp(math.floor(math.ldexp(float(d), bits - e)), e - bits)
    return hi, float(d - Decimal(hi))


def _split3(d: Decimal, bits: int) -> tuple[float, float, float]:
    hi, _ = _split(d, bits)
    mid, _ = _split(d - Decimal(hi), bits)
    return hi, mid, float(d - Decimal(hi) - Decimal(mid))


_LN2_HI, _LN2_LO = _split(_LN2, 32)
_INV_LN2 = float(1 / _LN2)
_PIO2_1, _PIO2_2, _PIO2_3 = _split3(_PI / 2, 33)
_TWO_OVER_PI = float(2 / _PI)
_PIO2, _PIO2_LO = float(_PI / 2), float(_PI / 2 - Decimal(float(_PI / 2)))
_PI_D, _PI_LO = float(_PI), float(_PI - Decimal(float(_PI)))
_SQRT_HALF = float(Decimal(2).sqrt() / 2)

_EXP_C = [float(Fraction(1, math.factorial(n))) for n in range(17)]           # 1/n!
_SIN_C = [float(Fraction((-1) ** n, math.factorial(2 * n + 1))) for n in range(11)]
_COS_C = [float(Fraction((-1) ** n, math.factorial(2 * n))) for n in range(11)]
_ATANH_C = [float(Fraction(1, 2 * n + 1)) for n in range(14)]                # 1/(2n+1)
_ATAN_C = [float(Fraction((-1) ** n, 2 * n + 1)) for n in range(15)]


def _horner(coefs, z):
    p = np.full_like(z, coefs[-1])
    for c in reversed(coefs[:-1]):
        p = p * z + c
    return p


def _f64(x):
    return np.asarray(x, dtype=np.float64)


def exp(x):
    """e**x for |x| < 700."""
    x = _f64(x)
    k = np.rint(x * _INV_LN2)
    r = (x - k * _LN2_HI) - k * _LN2_LO     # |r| <= ln2/2; k * _LN2_HI exact
    return np.ldexp(_horner(_EXP_C, r), k.astype(np.int64))


def log(x):
    """Natural logarithm of positive normal x."""
    x = _f64(x)
    m, e = np.frexp(x)                       # x = m 2**e, m in [0.5, 1)
    lo = m < _SQRT_HALF
    m = np.where(lo, m * 2.0, m)             # m in [sqrt(1/2), sqrt(2))
    e = (e - lo).astype(np.float64)
    f = m - 1.0                              # exact (Sterbenz)
    s = f / (2.0 + f)                        # log m = 2 atanh(s), |s| <= 0.1716
    lm = 2.0 * (s * _horner(_ATANH_C, s * s))
    return e * _LN2_HI + (lm + e * _LN2_LO)


def pow(x, y):
    """x**y for positive x, as exp(y log x)."""
    return exp(_f64(y) * log(x))


def _reduce_pio2(x):
    k = np.rint(x * _TWO_OVER_PI)
    r = ((x - k * _PIO2_1) - k * _PIO2_2) - k * _PIO2_3   # |r| <= pi/4 for |k| < 2**20
    return r, np.mod(k.astype(np.int64), 4)


def _sin_cos_reduced(r):
    z = r * r
    s = r + r * (z * _horner(_SIN_C[1:], z))
    c = _horner(_COS_C, z)
    return s, c


def sin(x):
    r, q = _reduce_pio2(_f64(x))
    s, c = _sin_cos_reduced(r)
    return np.select([q == 0, q == 1, q == 2], [s, c, -s], -c)


def cos(x):
    r, q = _reduce_pio2(_f64(x))
    s, c = _sin_cos_reduced(r)
    return np.select([q == 0, q == 1, q == 2], [c, -s, -c], s)


def _atan01(t):
    """arctan of t in [0, 1]: two half-angle steps, atan t = 2 atan(t / (1 + sqrt(1 + t^2))),
    bring t below tan(pi/16); then the series."""
    t = t / (1.0 + np.sqrt(1.0 + t * t))
    t = t / (1.0 + np.sqrt(1.0 + t * t))
    return 4.0 * (t * _horner(_ATAN_C, t * t))


def atan2(y, x):
    """Angle of (x, y) in [-pi, pi], with NumPy's signed-zero conventions."""
    y, x = np.broadcast_arrays(_f64(y), _f64(x))
    ay, ax = np.abs(y), np.abs(x)
    swap = ay > ax
    num = np.where(swap, ax, ay)
    den = np.where(swap, ay, ax)
    a = _atan01(num / np.where(den > 0, den, 1.0))
    a = np.where(swap, (_PIO2 - a) + _PIO2_LO, a)
    a = np.where(np.signbit(x), (_PI_D - a) + _PI_LO, a)
    return np.where(np.signbit(y), -a, a)


def atan(x):
    return atan2(_f64(x), np.ones_like(_f64(x)))


def asin(x):
    x = _f64(x)
    return atan2(x, np.sqrt((1.0 - x) * (1.0 + x)))


PI = _PI_D
