"""Particles (spheres) of the radial-lookup path, mirroring smuthi/particles.py:32-148."""
import functools

import numpy as np

from .linearsystem.tmatrix import t_matrix as tmt


class Particle:
    """Base particle: position [x, y, z], refractive index, multipole cut-offs."""

    def __init__(self, position=None, euler_angles=None, refractive_index=1 + 0j, l_max=None, m_max=None):
        self.position = list(position) if position is not None else [0, 0, 0]
        self.euler_angles = list(euler_angles) if euler_angles is not None else [0, 0, 0]
        self.refractive_index = refractive_index
        self.l_max = l_max
        self.m_max = m_max if m_max is not None else l_max
        self.initial_field = None
        self.scattered_field = None
        self.t_matrix = None


class Sphere(Particle):
    """Homogeneous sphere; its T-matrix is the diagonal Mie matrix."""

    def __init__(self, position=None, refractive_index=1 + 0j, radius=1, l_max=None, m_max=None):
        Particle.__init__(self, position=position, refractive_index=refractive_index, l_max=l_max, m_max=m_max)
        self.radius = radius

    def circumscribing_sphere_radius(self):
        return self.radius

    def is_outside(self, x, y, z):
        return ((x - self.position[0]) ** 2 + (y - self.position[1]) ** 2 + (z - self.position[2]) ** 2
                > self.radius ** 2)

    def compute_t_matrix(self, vacuum_wavelength, n_medium):
        return _sphere_t_matrix(self.radius, self.refractive_index, self.l_max, self.m_max, vacuum_wavelength,
                                n_medium)


@functools.lru_cache(maxsize=256)
def _sphere_t_matrix(radius, n_sphere, l_max, m_max, vacuum_wavelength, n_medium):
    omega = 2 * np.pi / vacuum_wavelength
    t = tmt.t_matrix_sphere(omega * n_medium, omega * n_sphere, radius, l_max, m_max)
    t.setflags(write=False)
    return t
