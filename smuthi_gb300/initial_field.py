"""Plane-wave initial field (smuthi/initial_field.py:66-106 and :272-329).

A plane wave is a discrete plane wave expansion (one in-plane wavenumber, one
azimuth). Its regular SWE at a particle is the closed-form PVWF -> SVWF
transformation (smuthi/fields/transformations.py:77-131 with one k point),
evaluated here for all particles at once.
"""
import numpy as np

from . import fields as flds
from . import layers as lay
from .fields.expansions import SphericalWaveExpansion
from .fields.transformations import transformation_coefficients_vwf
from .utility.math import legendre_normalized


class DiscretePWE:
    """Plane wave expansion with a single (kappa, alpha): g[pol] amplitudes."""

    def __init__(self, k, k_parallel, azimuthal_angle, kind, reference_z, g=None):
        self.k = k
        self.k_parallel = k_parallel
        self.azimuthal_angle = azimuthal_angle
        self.kind = kind
        self.reference_point = [0, 0, reference_z]
        self.coefficients = np.zeros(2, complex) if g is None else np.array(g, complex)

    def k_z(self):
        kz = flds.k_z(k_parallel=self.k_parallel, k=self.k)
        return kz if self.kind == 'upgoing' else -kz


class PlaneWave:
    """Plane wave of given polar / azimuthal propagation angle and polarization (0 TE, 1 TM).

    polar_angle < pi/2 travels upwards (incidence from the bottom layer),
    polar_angle > pi/2 downwards (incidence from the top layer).
    """

    def __init__(self, vacuum_wavelength, polar_angle, azimuthal_angle, polarization, amplitude=1,
                 reference_point=None):
        if polarization not in (0, 1):
            raise ValueError('polarization must be 0 (TE) or 1 (TM)')
        if np.isclose(np.cos(polar_angle), 0):
            raise ValueError('propagating waves not defined in the xy-plane')
        self.vacuum_wavelength = vacuum_wavelength
        self.polar_angle = polar_angle
        self.azimuthal_angle = azimuthal_angle
        self.polarization = polarization
        self.amplitude = amplitude
        self.reference_point = list(reference_point) if reference_point else [0, 0, 0]
        self.validity_conditions = []

    def angular_frequency(self):
        return flds.angular_frequency(self.vacuum_wavelength)

    def plane_wave_expansion(self, layer_system, i):
        """(upgoing, downgoing) discrete PWEs in layer i, including the layer response."""
        from_bottom = np.cos(self.polar_angle) > 0
        iP = 0 if from_bottom else layer_system.number_of_layers() - 1
        kind = 'upgoing' if from_bottom else 'downgoing'
        nP = layer_system.refractive_indices[iP]
        omega = self.angular_frequency()
        kP = nP * omega
        sp, cp = np.sin(self.polar_angle), np.cos(self.polar_angle)
        kx = kP * sp * np.cos(self.azimuthal_angle)
        ky = kP * sp * np.sin(self.azimuthal_angle)
        kz = kP * cp
        zP = layer_system.reference_z(iP)
        rp = self.reference_point
        amp = self.amplitude * np.exp(-1j * (kx * rp[0] + ky * rp[1] + kz * (rp[2] - zP)))
        kpar = sp * nP * omega
        g = np.zeros(2, complex)
        g[self.polarization] = amp
        k_i = omega * layer_system.refractive_indices[i]
        col = 0 if kind == 'upgoing' else 1
        up = DiscretePWE(k_i, kpar, self.azimuthal_angle, 'upgoing', layer_system.reference_z(i))
        down = DiscretePWE(k_i, kpar, self.azimuthal_angle, 'downgoing', layer_system.reference_z(i))
        for pol in range(2):
            L = lay.layersystem_response_matrix(pol, layer_system.thicknesses, layer_system.refractive_indices,
                                                kpar, omega, iP, i)[:, :, 0]
            up.coefficients[pol] = L[0, col] * g[pol]
            down.coefficients[pol] = L[1, col] * g[pol]
        if iP == i:
            (up if kind == 'upgoing' else down).coefficients += g
        return up, down

    def swe_coefficients(self, positions, layer_system, l_max, m_max):
        """Regular SWE coefficients [N, blocksize] of this wave about each position.

        All positions must lie in one layer.
        """
        positions = np.atleast_2d(np.asarray(positions, dtype=float))
        layer = layer_system.layer_number(positions[0, 2])
        tau, ll, mm = flds.index_table(l_max, m_max)
        out = np.zeros((len(positions), len(tau)), complex)
        for pwe in self.plane_wave_expansion(layer_system, layer):
            k = pwe.k
            kp = pwe.k_parallel
            a = pwe.azimuthal_angle
            kz = pwe.k_z()
            _, pilm, taulm = legendre_normalized(kz / k, kp / k, l_max)
            # per-n factor 4 sum_pol Bdag(n, pol) e^{-i m a} g_pol; the particle phase separates
            d = positions - np.array(pwe.reference_point)[None, :]
            ejkr = np.exp(1j * (kp * np.cos(a) * d[:, 0] + kp * np.sin(a) * d[:, 1] + kz * d[:, 2]))
            for n in range(len(tau)):
                acc = np.zeros(len(positions), complex)
                for pol in range(2):
                    bd = transformation_coefficients_vwf(tau[n], ll[n], mm[n], pol, pilm, taulm, dagger=True)[0]
                    acc += bd * (np.exp(-1j * mm[n] * a) * (pwe.coefficients[pol] * ejkr))
                out[:, n] += 4 * acc
        return out

    def spherical_wave_expansion(self, particle, layer_system):
        i = layer_system.layer_number(particle.position[2])
        swe = SphericalWaveExpansion(k=self.angular_frequency() * layer_system.refractive_indices[i],
                                     l_max=particle.l_max, m_max=particle.m_max, kind='regular',
                                     reference_point=particle.position, lower_z=layer_system.lower_zlimit(i),
                                     upper_z=layer_system.upper_zlimit(i))
        swe.coefficients = self.swe_coefficients([particle.position], layer_system, particle.l_max,
                                                 particle.m_max)[0]
        return swe
