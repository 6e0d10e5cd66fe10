"""Minimal spherical-wave-expansion container (smuthi/fields/expansions.py:242-463)."""
import numpy as np

from . import blocksize


class SphericalWaveExpansion:
    """Coefficients a_{tau l m} of a regular or outgoing SWE about a reference point."""

    def __init__(self, k, l_max, m_max=None, kind=None, reference_point=None, lower_z=-np.inf, upper_z=np.inf):
        self.k = k
        self.l_max = l_max
        self.m_max = l_max if m_max is None else m_max
        self.kind = kind
        self.reference_point = reference_point
        self.lower_z = lower_z
        self.upper_z = upper_z
        self.coefficients = np.zeros(blocksize(self.l_max, self.m_max), dtype=complex)
        self.validity_conditions = []

    def __add__(self, other):
        out = SphericalWaveExpansion(self.k, self.l_max, self.m_max, self.kind, self.reference_point,
                                     max(self.lower_z, other.lower_z), min(self.upper_z, other.upper_z))
        out.coefficients = self.coefficients + other.coefficients
        return out
