"""Elementwise transcendental functions built only from IEEE-754 +, -, *, /, sqrt and exact
scaling, so that the host-side case set-up (grid generation, geometry, parameters) gives
bit-identical inputs on every CPU architecture.  numpy's and libm's sin/cos/exp/pow are
vectorised differently on x86-64 and AArch64 and differ in the last ulp, which ten solver
iterations amplify to ~1e-9.

Methods (accuracy a few ulp, ample for grid generation):
  exp    Cody-Waite reduction by ln 2 (two-part constant) + Taylor polynomial of degree 13
  log    frexp to m in [sqrt(1/2), sqrt(2)), log m = 2 atanh((m-1)/(m+1)) by its series
  pow    exp(y log x) for x > 0
  sin/cos  reduction by pi/2 with a three-part constant + Taylor polynomials on [-pi/4, pi/4]
  atan2  two half-angle reductions atan t = 2 atan(t / (1 + sqrt(1 + t^2))) + atan series
All accept scalars or arrays and return float64 (0-d arrays become Python floats).
"""
from decimal import Decimal, getcontext

import numpy as np

getcontext().prec = 60
_PI_DEC = Decimal("3.14159265358979323846264338327950288419716939937510582097494")


def _split(value_dec, nbits):
    """Leading part of value with its mantissa cut to nbits bits (so k * part is exact for
    integers k below 2**(53-nbits)), and the decimal remainder."""
    v = float(value_dec)
    m, e = np.frexp(v)
    hi = float(np.ldexp(np.floor(m * 2.0 ** nbits), int(e) - nbits))
    return hi, value_dec - Decimal(hi)


_PIO2_1, _r = _split(_PI_DEC / 2, 33)
_PIO2_2, _r = _split(_r, 33)
_PIO2_3 = float(_r)
_PI = float(_PI_DEC)
_PIO2 = float(_PI_DEC / 2)
_TWO_OVER_PI = float(2 / _PI_DEC)
_LN2_DEC = Decimal("0.693147180559945309417232121458176568075500134360255254120680")
_LN2_HI, _r = _split(_LN2_DEC, 32)
_LN2_LO = float(_r)
_INV_LN2 = float(1 / _LN2_DEC)
_SQRT_HALF = float(Decimal(2).sqrt() / 2)


def _out(x, scalar):
    return float(x) if scalar else x


def _arr(x):
    a = np.asarray(x, dtype=np.float64)
    return a, a.ndim == 0


def exp(x):
    a, sc = _arr(x)
    k = np.rint(a * _INV_LN2)
    r = (a - k * _LN2_HI) - k * _LN2_LO
    p = np.ones_like(r)
    for n in range(13, 0, -1):          # Horner form of sum r^n / n!
        p = 1.0 + p * r / n
    return _out(np.ldexp(p, k.astype(np.int64)), sc)


def log(x):
    a, sc = _arr(x)
    m, e = np.frexp(a)
    small = m < _SQRT_HALF
    m = np.where(small, m * 2.0, m)
    e = np.where(small, e - 1, e).astype(np.float64)
    s = (m - 1.0) / (m + 1.0)
    s2 = s * s
    q = np.zeros_like(s)
    for n in range(23, 1, -2):          # 1/3 s^2 + 1/5 s^4 + ...
        q = (q + 1.0 / n) * s2
    lm = 2.0 * (s + s * q)
    return _out(e * _LN2_HI + (lm + e * _LN2_LO), sc)


def pow(x, y):
    a, sc = _arr(x)
    b = np.asarray(y, dtype=np.float64)
    return _out(exp(b * log(a)), sc and b.ndim == 0)


def _sin_poly(r):
    r2 = r * r
    p = np.zeros_like(r)
    for n in range(17, 1, -2):          # r - r^3/3! + r^5/5! - ...
        p = (1.0 - p) * r2 / ((n - 1) * n)
    return r * (1.0 - p)


def _cos_poly(r):
    r2 = r * r
    p = np.zeros_like(r)
    for n in range(18, 0, -2):          # 1 - r^2/2! + r^4/4! - ...
        p = (1.0 - p) * r2 / ((n - 1) * n)
    return 1.0 - p


def _reduce(a):
    k = np.rint(a * _TWO_OVER_PI)
    r = ((a - k * _PIO2_1) - k * _PIO2_2) - k * _PIO2_3
    return r, (k.astype(np.int64) & 3)


def sin(x):
    a, sc = _arr(x)
    r, q = _reduce(a)
    s, c = _sin_poly(r), _cos_poly(r)
    out = np.select([q == 0, q == 1, q == 2], [s, c, -s], -c)
    return _out(out, sc)


def cos(x):
    a, sc = _arr(x)
    r, q = _reduce(a)
    s, c = _sin_poly(r), _cos_poly(r)
    out = np.select([q == 0, q == 1, q == 2], [c, -s, -c], s)
    return _out(out, sc)


def _atan01(t):
    """atan(t) for 0 <= t <= 1."""
    for _ in range(2):
        t = t / (1.0 + np.sqrt(1.0 + t * t))
    t2 = t * t
    p = np.zeros_like(t)
    for n in range(31, 1, -2):          # t - t^3/3 + t^5/5 - ...
        p = (1.0 / n - p) * t2
    return 4.0 * (t - t * p)


def atan2(y, x):
    ya, s1 = _arr(y)
    xa, s2 = _arr(x)
    ya, xa = np.broadcast_arrays(ya, xa)
    ay, ax = np.abs(ya), np.abs(xa)
    big = ay > ax
    num = np.where(big, ax, ay)
    den = np.where(big, ay, ax)
    with np.errstate(invalid="ignore", divide="ignore"):
        t = np.where(den > 0, num / np.where(den > 0, den, 1.0), 0.0)
    a = _atan01(t)
    a = np.where(big, _PIO2 - a, a)
    a = np.where(xa < 0, _PI - a, a)
    a = np.where(ya < 0, -a, a)
    return _out(a, s1 and s2)


def hypot(x, y):
    a = np.asarray(x, dtype=np.float64)
    b = np.asarray(y, dtype=np.float64)
    r = np.sqrt(a * a + b * b)
    return _out(r, r.ndim == 0)


def radians(deg):
    return deg * (_PI / 180.0)


pi = _PI
