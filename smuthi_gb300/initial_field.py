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
        out = np.zeros((len(positions), flds.blocksize(l_max, m_max)), complex)
        for pwe in self.plane_wave_expansion(layer_system, layer):
            kr, amp = component_terms(pwe, l_max, m_max)
            # the per-n factor amp (4 sum_pol Bdag(n, pol) e^{-i m a} g_pol) and the particle phase separate
            d = positions - kr[4:7][None, :]
            ejkr = np.exp(1j * (kr[0] * d[:, 0] + kr[1] * d[:, 1] + complex(kr[2], kr[3]) * d[:, 2]))
            out += ejkr[:, None] * amp[None, :]
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


def component_terms(pwe, l_max, m_max):
    """Wavevector row and per-index factors of one discrete plane-wave component.

    Returns kr = [kx, ky, Re kz, Im kz, x0, y0, z0] (reference point r0) and amp[n] =
    4 sum_pol B^dagger(n, pol) e^{-i m alpha} g_pol, so that the component's regular SWE coefficient
    at a point r is amp[n] exp(i k . (r - r0)) (smuthi/fields/transformations.py:77-131, one k point).
    """
    k, kp, a = pwe.k, pwe.k_parallel, pwe.azimuthal_angle
    kz = complex(pwe.k_z())
    _, pilm, taulm = legendre_normalized(kz / k, kp / k, l_max)
    tau, ll, mm = flds.index_table(l_max, m_max)
    amp = np.zeros(len(tau), complex)
    for n in range(len(tau)):
        for pol in range(2):
            bd = transformation_coefficients_vwf(tau[n], ll[n], mm[n], pol, pilm, taulm, dagger=True)[0]
            amp[n] += 4 * bd * (np.exp(-1j * mm[n] * a) * pwe.coefficients[pol])
    kpr = float(np.real(kp))
    r0 = pwe.reference_point
    kr = np.array([kpr * np.cos(a), kpr * np.sin(a), kz.real, kz.imag, r0[0], r0[1], r0[2]], float)
    return kr, amp


def swe_coefficients_batch(fields, positions, layer_system, l_max, m_max, context):
    """Regular SWE coefficients [len(fields), N, blocksize] of plane waves at positions in one layer.

    The per-wave factors are formed here (O(blocksize) per plane-wave component); the particle-dependent
    part runs on the context's GPU (``sg_plane_wave_swe``, FP64). Falls back to the host for
    evanescent in-plane wavenumbers (complex k_parallel), which the kernel does not take.
    """
    import torch
    positions = np.atleast_2d(np.asarray(positions, dtype=float))
    layer = layer_system.layer_number(positions[0, 2])
    comps = [f.plane_wave_expansion(layer_system, layer) for f in fields]
    if any(np.iscomplexobj(c.k_parallel) and np.imag(c.k_parallel) != 0 for cs in comps for c in cs):
        return np.stack([f.swe_coefficients(positions, layer_system, l_max, m_max) for f in fields])
    nc = max(len(cs) for cs in comps)
    bs = flds.blocksize(l_max, m_max)
    kr = np.zeros((len(fields), nc, 7))
    amp = np.zeros((len(fields), nc, bs), complex)
    for q, cs in enumerate(comps):
        for c, pwe in enumerate(cs):
            kr[q, c], amp[q, c] = component_terms(pwe, l_max, m_max)
    dev = torch.device("cuda", context.device)
    xyz_t = torch.from_numpy(np.ascontiguousarray(positions)).to(dev)
    kr_t = torch.from_numpy(kr).to(dev)
    amp_t = torch.from_numpy(amp).to(dev)
    out_t = torch.empty((len(fields), len(positions), bs), dtype=torch.complex128, device=dev)
    context.plane_wave_swe_dev(len(positions), xyz_t.data_ptr(), len(fields), nc, kr_t.data_ptr(), bs,
                               amp_t.data_ptr(), out_t.data_ptr())
    return out_t.cpu().numpy()
