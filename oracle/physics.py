"""Oracle: Mie T-matrix, plane-wave RHS and the radial coupling lookup table.

Test infrastructure only; each function cites the reference code it restates.
"""
import numpy as np
import scipy.special

from . import layers as lay
from .special import (ab5_coefficients, angular_frequency, blocksize, dx_xh, dx_xj, index_triples, ipow, k_z,
                      legendre_normalized, multi_to_single_index, spherical_bessel, spherical_hankel,
                      transformation_coefficients_vwf)


class Sphere:
    """smuthi/particles.py:97-138 (position, refractive index, radius, l_max, m_max)."""

    def __init__(self, position, refractive_index, radius, l_max, m_max=None):
        self.position = list(position)
        self.refractive_index = refractive_index
        self.radius = radius
        self.l_max = l_max
        self.m_max = l_max if m_max is None else m_max


def mie_coefficient(tau, l, k_medium, k_particle, radius):
    """smuthi/linearsystem/tmatrix/t_matrix.py:8-38."""
    jm = spherical_bessel(l, k_medium * radius)
    jp = spherical_bessel(l, k_particle * radius)
    djm = dx_xj(l, k_medium * radius)
    djp = dx_xj(l, k_particle * radius)
    hm = spherical_hankel(l, k_medium * radius)
    dhm = dx_xh(l, k_medium * radius)
    if tau == 0:
        return (jm * djp - jp * djm) / (jp * dhm - hm * djp)
    return ((k_medium ** 2 * jm * djp - k_particle ** 2 * jp * djm)
            / (k_particle ** 2 * jp * dhm - k_medium ** 2 * hm * djp))


def t_matrix_sphere(k_medium, k_particle, radius, l_max, m_max):
    """smuthi/linearsystem/tmatrix/t_matrix.py:74-94 -- diagonal Mie T."""
    t = np.zeros((blocksize(l_max, m_max),) * 2, dtype=complex)
    for n, (tau, l, m) in enumerate(index_triples(l_max, m_max)):
        t[n, n] = mie_coefficient(tau, l, k_medium, k_particle, radius)
    return t


def particle_t_matrix(particle, vacuum_wavelength, layer_system):
    """smuthi/linearsystem/linear_system.py:135-147 + smuthi/particles.py:126-148."""
    n_med = layer_system.refractive_indices[layer_system.layer_number(particle.position[2])]
    w = 2 * np.pi / vacuum_wavelength
    return t_matrix_sphere(w * n_med, w * particle.refractive_index, particle.radius, particle.l_max, particle.m_max)


# --- plane wave initial field -----------------------------------------------

class PlaneWave:
    """smuthi/initial_field.py:272-329 (PlaneWave) + :66-95 (InitialPropagatingWave)."""

    def __init__(self, vacuum_wavelength, polar_angle, azimuthal_angle, polarization, amplitude=1,
                 reference_point=None):
        self.vacuum_wavelength = vacuum_wavelength
        self.polar_angle = polar_angle
        self.azimuthal_angle = azimuthal_angle
        self.polarization = polarization
        self.amplitude = amplitude
        self.reference_point = list(reference_point) if reference_point else [0, 0, 0]

    def plane_wave_expansion(self, ls, i):
        """smuthi/initial_field.py:284-329 -> ((kind, k, kpar, alpha, g[2]) up, ... down).

        A discrete plane wave expansion is held as a dict with keys ``k``,
        ``kpar`` (scalar), ``alpha`` (scalar), ``kind`` and ``g`` (2 pols).
        """
        if np.cos(self.polar_angle) > 0:
            iP, kind = 0, 'upgoing'
        else:
            iP, kind = ls.number_of_layers() - 1, 'downgoing'
        niP = ls.refractive_indices[iP]
        w = angular_frequency(self.vacuum_wavelength)
        neff = np.sin(self.polar_angle) * niP
        k_iP = niP * w
        kx = k_iP * np.sin(self.polar_angle) * np.cos(self.azimuthal_angle)
        ky = k_iP * np.sin(self.polar_angle) * np.sin(self.azimuthal_angle)
        kz = k_iP * np.cos(self.polar_angle)
        z_iP = ls.reference_z(iP)
        rp = self.reference_point
        amp = self.amplitude * np.exp(-1j * (kx * rp[0] + ky * rp[1] + kz * (rp[2] - z_iP)))
        g = np.zeros(2, complex)
        g[self.polarization] = amp
        exc = dict(k=k_iP, kpar=neff * w, alpha=self.azimuthal_angle, kind=kind, g=g, z=z_iP)
        up, down = layer_response(ls, exc, iP, i)
        if iP == i:
            if kind == 'upgoing':
                up['g'] = up['g'] + g
            else:
                down['g'] = down['g'] + g
        return up, down


def layer_response(ls, pwe, from_layer, to_layer):
    """smuthi/layers.py:141-191 for a discrete plane wave (one kpar, one alpha)."""
    w = pwe['k'] / ls.refractive_indices[from_layer]
    k_to = w * ls.refractive_indices[to_layer]
    z_to = ls.reference_z(to_layer)
    up = dict(k=k_to, kpar=pwe['kpar'], alpha=pwe['alpha'], kind='upgoing', g=np.zeros(2, complex), z=z_to)
    down = dict(k=k_to, kpar=pwe['kpar'], alpha=pwe['alpha'], kind='downgoing', g=np.zeros(2, complex), z=z_to)
    for pol in range(2):
        L = lay.response_matrix_scalar(pol, ls.thicknesses, ls.refractive_indices, pwe['kpar'], w,
                                       from_layer, to_layer)
        col = 0 if pwe['kind'] == 'upgoing' else 1
        up['g'][pol] = L[0, col] * pwe['g'][pol]
        down['g'][pol] = L[1, col] * pwe['g'][pol]
    return up, down


def pwe_to_swe(pwe, l_max, m_max, ref_point):
    """smuthi/fields/transformations.py:77-131 for a discrete plane wave."""
    k = pwe['k']
    kp = pwe['kpar']
    a = pwe['alpha']
    kz = k_z(kp, k) if pwe['kind'] == 'upgoing' else -k_z(kp, k)
    kvec = np.array([kp * np.cos(a), kp * np.sin(a), kz])
    d = np.array(ref_point) - np.array([0, 0, pwe['z']])
    ejkr = np.exp(1j * (kvec[0] * d[0] + kvec[1] * d[1] + kvec[2] * d[2]))
    _, pilm, taulm = legendre_normalized(kz / k, kp / k, l_max)
    coef = np.zeros(blocksize(l_max, m_max), complex)
    for n, (tau, l, m) in enumerate(index_triples(l_max, m_max)):
        acc = 0j
        for pol in range(2):
            bd = transformation_coefficients_vwf(tau, l, m, pol, pilm, taulm, dagger=True)[0]
            acc += bd * (np.exp(-1j * m * a) * (pwe['g'][pol] * ejkr))
        coef[n] = 4 * acc
    return coef


def initial_field_coefficients(initial_field, particle, ls):
    """smuthi/initial_field.py:92-106 -- regular SWE of the plane wave at a particle."""
    i = ls.layer_number(particle.position[2])
    up, down = initial_field.plane_wave_expansion(ls, i)
    return (pwe_to_swe(up, particle.l_max, particle.m_max, particle.position)
            + pwe_to_swe(down, particle.l_max, particle.m_max, particle.position))


# --- radial lookup table ------------------------------------------------------

def radial_coupling_lookup_table(vacuum_wavelength, particle_list, ls, k_parallel, resolution):
    """smuthi/linearsystem/particlecoupling/prepare_lookup.py:253-464.

    Returns (table[len_rho, B, B] complex, rho_grid). The direct part is held
    in complex64 exactly as the reference holds it (prepare_lookup.py:301)
    and promoted by adding the complex128 layer-mediated part (:459).
    """
    l_max = max(p.l_max for p in particle_list)
    m_max = max(p.m_max for p in particle_list)
    bs = blocksize(l_max, m_max)
    xy = np.array([p.position[:2] for p in particle_list], dtype=float)
    rho_pp = np.sqrt((xy[:, None, 0] - xy[None, :, 0]) ** 2 + (xy[:, None, 1] - xy[None, :, 1]) ** 2)
    rho = np.arange(-3 * resolution, rho_pp.max() + 3 * resolution, resolution)
    z = particle_list[0].position[2]
    i_s = ls.layer_number(z)
    k_is = ls.wavenumber(i_s, vacuum_wavelength)
    dz = z - ls.reference_z(i_s)
    nr = len(rho)
    trip = index_triples(l_max, m_max)

    # direct part (prepare_lookup.py:300-340)
    w = np.zeros((nr, bs, bs), dtype=np.complex64)
    hank = []
    for n in range(2 * l_max + 1):
        h = spherical_hankel(n, k_is * rho)
        h[rho <= 0] = np.nan
        hank.append(h)
    leg0, _, _ = legendre_normalized(np.array([0.0]), np.array([1.0]), 2 * l_max)
    for m1 in range(-m_max, m_max + 1):
        for m2 in range(-m_max, m_max + 1):
            dm = abs(m1 - m2)
            for l1 in range(max(1, abs(m1)), l_max + 1):
                for l2 in range(max(1, abs(m2)), l_max + 1):
                    A = np.zeros(nr, complex)
                    B = np.zeros(nr, complex)
                    for ld in range(max(abs(l1 - l2), dm), l1 + l2 + 1):
                        a5, b5 = ab5_coefficients(l2, m2, l1, m1, ld)
                        A = A + a5 * hank[ld] * leg0[ld, dm]
                        B = B + b5 * hank[ld] * leg0[ld, dm]
                    for t1 in range(2):
                        n1 = multi_to_single_index(t1, l1, m1, l_max, m_max)
                        for t2 in range(2):
                            n2 = multi_to_single_index(t2, l2, m2, l_max, m_max)
                            w[:, n1, n2] = A if t1 == t2 else B
    offdiag = rho_pp[~np.eye(len(particle_list), dtype=bool)]
    w[rho < offdiag.min() / 2, :, :] = 0

    if ls.is_degenerate():
        return w, rho

    # layer-mediated part (prepare_lookup.py:343-459)
    kp = np.asarray(k_parallel)
    kz = k_z(kp, k_is)
    epl = np.exp(2j * kz * dz)
    emn = np.exp(-2j * kz * dz)
    omega = angular_frequency(vacuum_wavelength)
    L = np.zeros((2, 2, 2, len(kp)), complex)
    for pol in range(2):
        L[pol] = lay.response_matrix(pol, ls.thicknesses, ls.refractive_indices, kp, omega, i_s, i_s)
    ct = kz / k_is
    st = kp / k_is
    _, pi_pl, tau_pl = legendre_normalized(ct, st, l_max)
    _, pi_mn, tau_mn = legendre_normalized(-ct, st, l_max)
    Bd = np.zeros((2, 2, bs, len(kp)), complex)
    Bn = np.zeros((2, 2, bs, len(kp)), complex)
    m_of = [t[2] for t in trip]
    for n, (tau, l, m) in enumerate(trip):
        for pol in range(2):
            Bd[pol, 0, n] = transformation_coefficients_vwf(tau, l, m, pol, pi_pl, tau_pl, dagger=True)
            Bd[pol, 1, n] = transformation_coefficients_vwf(tau, l, m, pol, pi_mn, tau_mn, dagger=True)
            Bn[pol, 0, n] = transformation_coefficients_vwf(tau, l, m, pol, pi_pl, tau_pl, dagger=False)
            Bn[pol, 1, n] = transformation_coefficients_vwf(tau, l, m, pol, pi_mn, tau_mn, dagger=False)
    dkp = np.diff(kp)
    wr = np.zeros((nr, bs, bs), complex)
    for dm in range(2 * m_max + 1):
        besjac = scipy.special.jv(dm, kp[None, :] * rho[:, None]) * (kp / (kz * k_is))[None, :]
        for n1 in range(bs):
            for n2 in range(bs):
                if abs(m_of[n1] - m_of[n2]) != dm:
                    continue
                belbe = np.zeros(len(kp), complex)
                for pol in range(2):
                    belbe += L[pol, 0, 0] * Bd[pol, 0, n1] * Bn[pol, 0, n2]
                    belbe += L[pol, 1, 0] * Bd[pol, 1, n1] * Bn[pol, 0, n2] * emn
                    belbe += L[pol, 0, 1] * Bd[pol, 0, n1] * Bn[pol, 1, n2] * epl
                    belbe += L[pol, 1, 1] * Bd[pol, 1, n1] * Bn[pol, 1, n2]
                f = besjac * belbe[None, :]
                wr[:, n1, n2] = 2 * ipow(abs(m_of[n2] - m_of[n1])) * ((f[:, :-1] + f[:, 1:]) * dkp[None, :]).sum(-1)
    return w + wr, rho
