"""SVWF <-> PVWF transformation coefficients and SVWF translation coefficients.

``transformation_coefficients_vwf`` follows smuthi/fields/transformations.py:18-74;
``ab5_coefficients`` follows :414-447 (the a5/b5 translation coefficients).
"""
import functools

import numpy as np

from ..utility.math import wigner3j

_IPOW = (1 + 0j, 1j, -1 + 0j, -1j)


def ipow(k):
    """Exact i**k for integer k."""
    return _IPOW[k % 4]


def transformation_coefficients_vwf(tau, l, m, pol, pilm_list, taulm_list, dagger=False):
    """B_{tau l m, pol} (dagger: PVWF -> SVWF expansion, else SVWF -> PVWF)."""
    ang = taulm_list[l, abs(m)] if tau == pol else m * pilm_list[l, abs(m)]
    unit = -1j if dagger else 1j
    pre = -1 / unit ** (l + 1) / np.sqrt(2 * l * (l + 1))
    if pol == 0:
        pre = pre * unit
    return pre * ang


@functools.lru_cache(maxsize=None)
def ab5_coefficients(l1, m1, l2, m2, p):
    """(a5, b5) coefficients of the SVWF addition theorem."""
    jfac = ipow(abs(m1 - m2) - abs(m1) - abs(m2) + l2 - l1 + p) * (-1) ** (m1 - m2)
    fac1 = np.sqrt((2 * l1 + 1) * (2 * l2 + 1) / (2 * l1 * (l1 + 1) * l2 * (l2 + 1)))
    fac2a = (l1 * (l1 + 1) + l2 * (l2 + 1) - p * (p + 1)) * np.sqrt(2 * p + 1)
    fac2b = np.sqrt((l1 + l2 + 1 + p) * (l1 + l2 + 1 - p) * (p + l1 - l2) * (p - l1 + l2) * (2 * p + 1))
    w1 = wigner3j(l1, l2, p, m1, -m2, -(m1 - m2))
    w2a = wigner3j(l1, l2, p, 0, 0, 0)
    w2b = wigner3j(l1, l2, p - 1, 0, 0, 0)
    return jfac * fac1 * fac2a * w1 * w2a, jfac * fac1 * fac2b * w1 * w2b
