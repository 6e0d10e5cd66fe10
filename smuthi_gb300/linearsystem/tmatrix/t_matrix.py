"""Mie T-matrix of a sphere (smuthi/linearsystem/tmatrix/t_matrix.py:8-94)."""
import numpy as np

from ... import fields as flds
from ...utility import math as sf


def mie_coefficient(tau, l, k_medium, k_particle, radius):
    """Mie coefficient q_{tau l} (tau 0: spherical TE, 1: spherical TM)."""
    xm = k_medium * radius
    xp = k_particle * radius
    jm, jp = sf.spherical_bessel(l, xm), sf.spherical_bessel(l, xp)
    djm, djp = sf.dx_xj(l, xm), sf.dx_xj(l, xp)
    hm, dhm = sf.spherical_hankel(l, xm), sf.dx_xh(l, xm)
    if tau == 0:
        return (jm * djp - jp * djm) / (jp * dhm - hm * djp)
    if tau == 1:
        km2, kp2 = k_medium ** 2, k_particle ** 2
        return (km2 * jm * djp - kp2 * jp * djm) / (kp2 * jp * dhm - km2 * hm * djp)
    raise ValueError('tau must be 0 (spherical TE) or 1 (spherical TM)')


def t_matrix_sphere(k_medium, k_particle, radius, l_max, m_max):
    """Diagonal blocksize x blocksize T-matrix of a sphere."""
    tau, ll, mm = flds.index_table(l_max, m_max)
    q = {}
    for t in range(2):
        for l in range(1, l_max + 1):
            q[t, l] = mie_coefficient(t, l, k_medium, k_particle, radius)
    return np.diag(np.array([q[t, l] for t, l in zip(tau, ll)], dtype=complex))
