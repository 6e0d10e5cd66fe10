"""Oracle: indexing, contours and special functions of the reference.

Each function restates the cited reference function (paths relative to the
reference project root). Test infrastructure only.
"""
import math
from fractions import Fraction

import numpy as np
import scipy.special

_I_POW = (1 + 0j, 1j, -1 + 0j, -1j)


def ipow(k):
    """Exact integer power of the imaginary unit, i**k."""
    return _I_POW[k % 4]


def angular_frequency(vacuum_wavelength):
    """smuthi/fields/__init__.py:12-22 (omega = 2 pi / lambda, c = 1)."""
    return 2 * np.pi / vacuum_wavelength


def multi_to_single_index(tau, l, m, l_max, m_max):
    """smuthi/fields/__init__.py:29-80 -- SVWF multi index n(tau, l, m)."""
    tau_blocksize = m_max * (m_max + 2) + (l_max - m_max) * (2 * m_max + 1)
    n = tau * tau_blocksize
    if (l - 1) <= m_max:
        n += (l - 1) * (l + 1)
    else:
        n += m_max * (m_max + 2) + (l - 1 - m_max) * (2 * m_max + 1)
    return n + m + min(l, m_max)


def blocksize(l_max, m_max):
    """smuthi/fields/__init__.py:83-94."""
    return multi_to_single_index(1, l_max, m_max, l_max, m_max) + 1


def index_triples(l_max, m_max):
    """List of (tau, l, m) in multi-index order for one particle."""
    out = [None] * blocksize(l_max, m_max)
    for tau in range(2):
        for l in range(1, l_max + 1):
            for m in range(-min(l, m_max), min(l, m_max) + 1):
                out[multi_to_single_index(tau, l, m, l_max, m_max)] = (tau, l, m)
    return out


def k_z(k_parallel, k):
    """smuthi/fields/__init__.py:101-129 -- sqrt(k^2 - kappa^2), Im >= 0."""
    kz = np.sqrt(k ** 2 - np.asarray(k_parallel) ** 2 + 0j)
    return np.where(kz.imag < 0, -kz, kz)


# --- Sommerfeld contour ------------------------------------------------------

def reasonable_neff_waypoints(layer_refractive_indices, neff_imag=1e-2, neff_max=None, neff_max_offset=1):
    """smuthi/fields/__init__.py:153-194."""
    nr = np.array(layer_refractive_indices).real
    lo = max(0, min(nr) - 0.1)
    hi = max(nr) + 0.2
    if neff_max is None:
        neff_max = hi + neff_max_offset
    if neff_imag == 0:
        return [0, neff_max]
    wp = [0, lo, lo - 1j * neff_imag, hi - 1j * neff_imag, hi]
    if neff_max > hi:
        wp.append(neff_max)
    return wp


def create_neff_array(neff_waypoints, neff_resolution):
    """smuthi/fields/__init__.py:197-216 -- piecewise-linear contour samples."""
    segs = []
    for a, b in zip(neff_waypoints[:-1], neff_waypoints[1:]):
        if abs(b - a) > 0:
            num = int(np.ceil(abs(b - a) / neff_resolution)) + 1
            segs.append(a + np.linspace(0, 1, num=num, endpoint=True, dtype=complex) * (b - a))
    return np.concatenate(segs)


def branchpoint_correction(layer_refractive_indices, neff, min_dist):
    """smuthi/fields/__init__.py:239-273 -- move samples off branch points."""
    for n in layer_refractive_indices:
        while True:
            hits = np.where(abs(neff - n) < min_dist)[0]
            if len(hits) == 0:
                break
            idx = hits[0]
            if idx != len(neff) - 1:
                neff = np.insert(neff, idx + 1, (neff[idx] + neff[idx + 1]) / 2.0)
                if abs(neff[idx + 1] - n) < min_dist:
                    neff = np.delete(neff, idx + 1)
            if idx != 0:
                neff[idx] = (neff[idx - 1] + neff[idx]) / 2.0
                if abs(neff[idx] - n) < min_dist:
                    neff = np.delete(neff, idx)
    return neff


def sommerfeld_kpar_contour(vacuum_wavelength, layer_refractive_indices, neff_waypoints=None, neff_imag=1e-2,
                            neff_max=None, neff_max_offset=1, neff_resolution=1e-2,
                            neff_minimal_branchpoint_distance=None):
    """smuthi/fields/__init__.py:276-370 (reasonable_Sommerfeld_kpar_contour)."""
    if neff_waypoints is None:
        neff_waypoints = reasonable_neff_waypoints(layer_refractive_indices, neff_imag, neff_max, neff_max_offset)
    if neff_minimal_branchpoint_distance is None:
        neff_minimal_branchpoint_distance = neff_resolution / 5
    neff = create_neff_array(neff_waypoints, neff_resolution)
    if layer_refractive_indices is not None:
        neff = branchpoint_correction(layer_refractive_indices, neff, neff_minimal_branchpoint_distance)
    return neff * angular_frequency(vacuum_wavelength)


def angular_arrays(angular_resolution=np.pi / 360):
    """smuthi/fields/__init__.py:132-136 -> (azimuthal, polar)."""
    az = np.arange(0, 2 * np.pi + 0.5 * angular_resolution, angular_resolution, dtype=float)
    po = np.arange(0, np.pi + 0.5 * angular_resolution, angular_resolution, dtype=float)
    return az, po


# --- special functions -------------------------------------------------------

def _legendre_prefactor(m):
    """smuthi/utility/numba_helpers.py:81-94 (m <= 10 branch of prefactor_expansion)."""
    res = 1.0
    for t in range(2, 2 * m + 2, 2):
        res += res / t
    return (res / 2) ** 0.5


def legendre_normalized(ct, st, lmax):
    """smuthi/utility/math.py:38-104 -- normalized P_l^m, pi_l^m, tau_l^m.

    Returns three complex arrays indexed [l, m, *ct.shape].
    """
    ct = np.atleast_1d(np.asarray(ct, dtype=np.complex128))
    st = np.atleast_1d(np.asarray(st, dtype=np.complex128))
    shp = (lmax + 1, lmax + 1) + ct.shape
    plm = np.zeros(shp, complex)
    pilm = np.zeros(shp, complex)
    taulm = np.zeros(shp, complex)
    dp0 = np.zeros((lmax + 1,) + ct.shape, complex)
    plm[0, 0] = np.sqrt(2) / 2
    if lmax >= 1:
        plm[1, 0] = np.sqrt(3 / 2) * ct
        dp0[1] = np.sqrt(3) * plm[0, 0]
        taulm[1, 0] = -st * dp0[1]
    taulm[0, 0] = -st * dp0[0]
    for l in range(1, lmax):
        plm[l + 1, 0] = (1 / (l + 1) * np.sqrt((2 * l + 1) * (2 * l + 3)) * ct * plm[l, 0]
                         - l / (l + 1) * np.sqrt((2 * l + 3) / (2 * l - 1)) * plm[l - 1, 0])
        dp0[l + 1] = ((l + 1) * np.sqrt((2 * (l + 1) + 1) / (2 * (l + 1) - 1)) * plm[l, 0]
                      + np.sqrt((2 * (l + 1) + 1) / (2 * (l + 1) - 1)) * ct * dp0[l])
        taulm[l + 1, 0] = -st * dp0[l + 1]
    for m in range(1, lmax + 1):
        pf = _legendre_prefactor(m)
        plm[m, m] = pf * st ** m
        pilm[m, m] = pf * st ** (m - 1)
        taulm[m, m] = m * ct * pilm[m, m]
        for l in range(m, lmax):
            c1 = np.sqrt((2 * l + 1) * (2 * l + 3) / ((l + 1 - m) * (l + 1 + m)))
            c2 = np.sqrt((2 * l + 3) * (l - m) * (l + m) / ((2 * l - 1) * (l + 1 - m) * (l + 1 + m)))
            plm[l + 1, m] = c1 * ct * plm[l, m] - c2 * plm[l - 1, m]
            c1p = np.sqrt((2 * l + 1) * (2 * l + 3) / (l + 1 - m) / (l + 1 + m))
            c2p = np.sqrt((2 * l + 3) * (l - m) * (l + m) / (2 * l - 1) / (l + 1 - m) / (l + 1 + m))
            pilm[l + 1, m] = c1p * ct * pilm[l, m] - c2p * pilm[l - 1, m]
            taulm[l + 1, m] = ((l + 1) * ct * pilm[l + 1, m]
                               - (l + 1 + m) * np.sqrt((2 * (l + 1) + 1) * (l + 1 - m) / (2 * (l + 1) - 1)
                                                       / (l + 1 + m)) * pilm[l, m])
    return plm, pilm, taulm


def spherical_hankel(n, x):
    """smuthi/utility/math.py:110-115 -- h_n^(1)(x) = j_n + i y_n (y_n(0) -> nan)."""
    x = np.asarray(x)
    yn = scipy.special.spherical_yn(n, x)
    if yn.ndim:
        yn = np.where(x == 0, np.nan, yn)
    return scipy.special.spherical_jn(n, x) + 1j * yn


def spherical_bessel(n, x):
    """smuthi/utility/math.py:107."""
    return scipy.special.spherical_jn(n, x)


def dx_xj(n, x):
    """smuthi/utility/math.py:118-129."""
    return x * spherical_bessel(n - 1, x) - n * spherical_bessel(n, x)


def dx_xh(n, x):
    """smuthi/utility/math.py:132-143."""
    return x * spherical_hankel(n - 1, x) - n * spherical_hankel(n, x)


def wigner3j(j1, j2, j3, m1, m2, m3):
    """Wigner 3j symbol (integer j, m) by the exact Racah formula.

    The reference evaluates ``sympy.physics.wigner.wigner_3j`` (fallback at
    smuthi/utility/math.py:26-35, pywigxjpf being absent); this restates the
    same closed form with exact rationals and rounds once to float.
    """
    if m1 + m2 + m3 != 0:
        return 0.0
    if min(j1, j2, j3) < 0 or abs(m1) > j1 or abs(m2) > j2 or abs(m3) > j3:
        return 0.0
    if j1 + j2 - j3 < 0 or j1 - j2 + j3 < 0 or -j1 + j2 + j3 < 0:
        return 0.0
    f = math.factorial
    tri = Fraction(f(j1 + j2 - j3) * f(j1 - j2 + j3) * f(-j1 + j2 + j3), f(j1 + j2 + j3 + 1))
    rad = tri * f(j1 + m1) * f(j1 - m1) * f(j2 + m2) * f(j2 - m2) * f(j3 + m3) * f(j3 - m3)
    kmin = max(0, j2 - j3 - m1, j1 - j3 + m2)
    kmax = min(j1 + j2 - j3, j1 - m1, j2 + m2)
    s = Fraction(0)
    for k in range(kmin, kmax + 1):
        den = (f(k) * f(j1 + j2 - j3 - k) * f(j1 - m1 - k) * f(j2 + m2 - k)
               * f(j3 - j2 + m1 + k) * f(j3 - j1 - m2 + k))
        s += Fraction((-1) ** k, den)
    sign = -1 if (j1 - j2 - m3) % 2 else 1
    if s == 0:
        return 0.0
    # value = sign * s * sqrt(rad); evaluate sqrt(s^2 * rad) exactly-rational then one sqrt
    val2 = s * s * rad
    mag = math.sqrt(val2.numerator) / math.sqrt(val2.denominator)
    return float(sign * (1 if s > 0 else -1) * mag)


_AB5_CACHE = {}


def ab5_coefficients(l1, m1, l2, m2, p):
    """smuthi/fields/transformations.py:414-447 -- SVWF translation a5, b5."""
    key = (l1, m1, l2, m2, p)
    if key in _AB5_CACHE:
        return _AB5_CACHE[key]
    jfac = ipow(abs(m1 - m2) - abs(m1) - abs(m2) + l2 - l1 + p) * (-1) ** (m1 - m2)
    fac1 = np.sqrt((2 * l1 + 1) * (2 * l2 + 1) / (2 * l1 * (l1 + 1) * l2 * (l2 + 1)))
    fac2a = (l1 * (l1 + 1) + l2 * (l2 + 1) - p * (p + 1)) * np.sqrt(2 * p + 1)
    fac2b = np.sqrt((l1 + l2 + 1 + p) * (l1 + l2 + 1 - p) * (p + l1 - l2) * (p - l1 + l2) * (2 * p + 1))
    wig1 = wigner3j(l1, l2, p, m1, -m2, -(m1 - m2))
    wig2a = wigner3j(l1, l2, p, 0, 0, 0)
    wig2b = wigner3j(l1, l2, p - 1, 0, 0, 0)
    a = jfac * fac1 * fac2a * wig1 * wig2a
    b = jfac * fac1 * fac2b * wig1 * wig2b
    _AB5_CACHE[key] = (a, b)
    return a, b


def transformation_coefficients_vwf(tau, l, m, pol, pilm, taulm, dagger=False):
    """smuthi/fields/transformations.py:18-74 -- SVWF<->PVWF coefficient B."""
    sphfun = taulm[l, abs(m)] if tau == pol else m * pilm[l, abs(m)]
    base = (-1j) if dagger else 1j
    prefac = -1 / base ** (l + 1) / np.sqrt(2 * l * (l + 1))
    if pol == 0:
        prefac = prefac * base
    return prefac * sphfun
