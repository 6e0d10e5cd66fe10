"""Special functions for the host-side preparation (FP64).

Normalized associated Legendre functions with the pi/tau angular functions
(smuthi/utility/math.py:38-104), spherical Bessel/Hankel functions and their
Riccati derivatives (:107-143), and exact Wigner 3j symbols (the reference
evaluates sympy's ``wigner_3j``, :26-35; here the Racah closed form over
exact rationals is rounded once to float).
"""
import functools
import math
from fractions import Fraction

import numpy as np
import scipy.special


def _pmm_prefactor(m):
    # sqrt((2m+1)!! / (2 (2m)!!)) built multiplicatively to keep full precision
    acc = 1.0
    for t in range(2, 2 * m + 2, 2):
        acc += acc / t
    return (acc / 2) ** 0.5


def legendre_normalized(ct, st, lmax):
    """Return (P_l^m, pi_l^m, tau_l^m) as complex arrays [l, m, *ct.shape]."""
    ct = np.atleast_1d(np.asarray(ct, dtype=np.complex128))
    st = np.atleast_1d(np.asarray(st, dtype=np.complex128))
    shape = (lmax + 1, lmax + 1) + ct.shape
    P = np.zeros(shape, complex)
    PI = np.zeros(shape, complex)
    TAU = np.zeros(shape, complex)
    dP0 = np.zeros((lmax + 1,) + ct.shape, complex)
    P[0, 0] = np.sqrt(2) / 2
    if lmax >= 1:
        P[1, 0] = np.sqrt(3 / 2) * ct
        dP0[1] = np.sqrt(3) * P[0, 0]
        TAU[1, 0] = -st * dP0[1]
    for l in range(1, lmax):
        P[l + 1, 0] = (1 / (l + 1) * np.sqrt((2 * l + 1) * (2 * l + 3)) * ct * P[l, 0]
                       - l / (l + 1) * np.sqrt((2 * l + 3) / (2 * l - 1)) * P[l - 1, 0])
        f = np.sqrt((2 * (l + 1) + 1) / (2 * (l + 1) - 1))
        dP0[l + 1] = (l + 1) * f * P[l, 0] + f * ct * dP0[l]
        TAU[l + 1, 0] = -st * dP0[l + 1]
    for m in range(1, lmax + 1):
        pf = _pmm_prefactor(m)
        P[m, m] = pf * st ** m
        PI[m, m] = pf * st ** (m - 1)
        TAU[m, m] = m * ct * PI[m, m]
        for l in range(m, lmax):
            a = np.sqrt((2 * l + 1) * (2 * l + 3) / ((l + 1 - m) * (l + 1 + m)))
            b = np.sqrt((2 * l + 3) * (l - m) * (l + m) / ((2 * l - 1) * (l + 1 - m) * (l + 1 + m)))
            P[l + 1, m] = a * ct * P[l, m] - b * P[l - 1, m]
            a2 = np.sqrt((2 * l + 1) * (2 * l + 3) / (l + 1 - m) / (l + 1 + m))
            b2 = np.sqrt((2 * l + 3) * (l - m) * (l + m) / (2 * l - 1) / (l + 1 - m) / (l + 1 + m))
            PI[l + 1, m] = a2 * ct * PI[l, m] - b2 * PI[l - 1, m]
            c = (l + 1 + m) * np.sqrt((2 * (l + 1) + 1) * (l + 1 - m) / (2 * (l + 1) - 1) / (l + 1 + m))
            TAU[l + 1, m] = (l + 1) * ct * PI[l + 1, m] - c * PI[l, m]
    return P, PI, TAU


def spherical_bessel(n, x):
    return scipy.special.spherical_jn(n, x)


def spherical_hankel(n, x):
    """Spherical Hankel function of the first kind, h_n = j_n + i y_n (nan at x == 0)."""
    x = np.asarray(x)
    y = scipy.special.spherical_yn(n, x)
    if y.ndim:
        y = np.where(x == 0, np.nan, y)
    return scipy.special.spherical_jn(n, x) + 1j * y


def dx_xj(n, x):
    return x * spherical_bessel(n - 1, x) - n * spherical_bessel(n, x)


def dx_xh(n, x):
    return x * spherical_hankel(n - 1, x) - n * spherical_hankel(n, x)


@functools.lru_cache(maxsize=None)
def wigner3j(j1, j2, j3, m1, m2, m3):
    """Wigner 3j symbol for integer arguments (0 outside the selection rules)."""
    if m1 + m2 + m3 != 0 or min(j1, j2, j3) < 0:
        return 0.0
    if abs(m1) > j1 or abs(m2) > j2 or abs(m3) > j3:
        return 0.0
    a, b, c = j1 + j2 - j3, j1 - j2 + j3, -j1 + j2 + j3
    if min(a, b, c) < 0:
        return 0.0
    f = math.factorial
    total = Fraction(0)
    for k in range(max(0, j2 - j3 - m1, j1 - j3 + m2), min(a, j1 - m1, j2 + m2) + 1):
        total += Fraction((-1) ** k, f(k) * f(a - k) * f(j1 - m1 - k) * f(j2 + m2 - k) * f(j3 - j2 + m1 + k)
                          * f(j3 - j1 - m2 + k))
    if total == 0:
        return 0.0
    sq = Fraction(f(a) * f(b) * f(c) * f(j1 + m1) * f(j1 - m1) * f(j2 + m2) * f(j2 - m2) * f(j3 + m3) * f(j3 - m3),
                  f(j1 + j2 + j3 + 1))
    v2 = total * total * sq
    mag = math.sqrt(v2.numerator) / math.sqrt(v2.denominator)
    sign = (-1) ** ((j1 - j2 - m3) % 2) * (1 if total > 0 else -1)
    return float(sign * mag)
