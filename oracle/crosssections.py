"""Oracle: extinction and total scattering cross sections of a plane wave.

Restates smuthi/postprocessing/far_field.py:429-654 with
smuthi/postprocessing/scattered_field.py:80-150 and
smuthi/fields/transformations.py:133-233. Test infrastructure only.
"""
import numpy as np

from . import layers as lay
from .special import (angular_arrays, angular_frequency, index_triples, k_z, legendre_normalized,
                      transformation_coefficients_vwf)


def _swe_to_pwe(coef, l_max, m_max, k, pos, ls, kpar, alpha, layer_number=None, mediated=False):
    """transformations.py:133-226 -> (g_up, g_down) arrays [2, len(kpar), len(alpha)]."""
    kpar = np.atleast_1d(np.asarray(kpar))
    alpha = np.atleast_1d(np.asarray(alpha))
    i_swe = ls.layer_number(pos[2])
    if layer_number is None and not mediated:
        layer_number = i_swe
    ref = [0, 0, ls.reference_z(i_swe)]
    kpg, ag = np.meshgrid(kpar, alpha, indexing='ij')
    kx = kpg * np.cos(ag)
    ky = kpg * np.sin(ag)
    kzu = k_z(kpg, k)
    kzd = -kzu
    kzvec = k_z(kpar, k)
    r = np.array(ref) - np.array(pos)
    eu = np.exp(1j * (kx * r[0] + ky * r[1] + kzu * r[2]))
    ed = np.exp(1j * (kx * r[0] + ky * r[1] + kzd * r[2]))
    _, pi_u, ta_u = legendre_normalized(kzvec / k, kpar / k, l_max)
    _, pi_d, ta_d = legendre_normalized(-kzvec / k, kpar / k, l_max)
    gu = np.zeros((2, len(kpar), len(alpha)), complex)
    gd = np.zeros((2, len(kpar), len(alpha)), complex)
    nidx = {t: n for n, t in enumerate(index_triples(l_max, m_max))}
    for m in range(-m_max, m_max + 1):
        eima = np.exp(1j * m * alpha)
        for pol in range(2):
            bu = np.zeros(len(kpar), complex)
            bd = np.zeros(len(kpar), complex)
            for l in range(max(1, abs(m)), l_max + 1):
                for tau in range(2):
                    c = coef[nidx[(tau, l, m)]]
                    bu += c * transformation_coefficients_vwf(tau, l, m, pol, pi_u, ta_u)
                    bd += c * transformation_coefficients_vwf(tau, l, m, pol, pi_d, ta_d)
            gu[pol] += bu[:, None] * eima[None, :]
            gd[pol] += bd[:, None] * eima[None, :]
    gu = gu / (2 * np.pi * kzvec[None, :, None] * k) * eu[None]
    gd = gd / (2 * np.pi * kzvec[None, :, None] * k) * ed[None]
    if mediated:
        omega = k / ls.refractive_indices[i_swe]
        ru = np.zeros_like(gu)
        rd = np.zeros_like(gd)
        for pol in range(2):
            L = lay.response_matrix(pol, ls.thicknesses, ls.refractive_indices, kpar, omega, i_swe, layer_number)
            ru[pol] = L[0, 0][:, None] * gu[pol] + L[0, 1][:, None] * gd[pol]
            rd[pol] = L[1, 0][:, None] * gu[pol] + L[1, 1][:, None] * gd[pol]
        return ru, rd
    return gu, gd


def scattered_field_pwe(vacuum_wavelength, particles, coefs, ls, layer_number, kpar, alpha):
    """scattered_field.py:80-150 (direct + layer-mediated, all particles)."""
    kpar = np.atleast_1d(np.asarray(kpar))
    alpha = np.atleast_1d(np.asarray(alpha))
    omega = angular_frequency(vacuum_wavelength)
    gu = np.zeros((2, len(kpar), len(alpha)), complex)
    gd = np.zeros_like(gu)
    for p, c in zip(particles, coefs):
        i_p = ls.layer_number(p.position[2])
        k = omega * ls.refractive_indices[i_p]
        if i_p == layer_number:
            u, d = _swe_to_pwe(c, p.l_max, p.m_max, k, p.position, ls, kpar, alpha)
            gu += u
            gd += d
        u, d = _swe_to_pwe(c, p.l_max, p.m_max, k, p.position, ls, kpar, alpha, layer_number, mediated=True)
        gu += u
        gd += d
    return gu, gd


def extinction_cross_section(initial_field, particles, coefs, ls):
    """far_field.py:517-654 with extinction_direction='both'."""
    i_top = ls.number_of_layers() - 1
    lam = initial_field.vacuum_wavelength
    omega = angular_frequency(lam)
    k_bot = omega * ls.refractive_indices[0]
    k_top = omega * ls.refractive_indices[-1]
    pol_P = initial_field.polarization
    beta = initial_field.polar_angle
    alpha = initial_field.azimuthal_angle
    if np.cos(beta) > 0:
        i_P, n_P, k_P = 0, ls.refractive_indices[0], k_bot
    else:
        i_P, n_P, k_P = i_top, ls.refractive_indices[i_top], k_top
    n_P = np.real(n_P)
    kappa = np.sin(beta) * k_P
    kvec = np.array([np.cos(alpha) * kappa, np.sin(alpha) * kappa, k_P * np.cos(beta)])
    rvec = np.array([0, 0, ls.reference_z(i_P)]) - np.array(initial_field.reference_point)
    A_P = initial_field.amplitude * np.exp(1j * np.dot(kvec, rvec))
    I0 = abs(A_P) ** 2 * n_P / 2
    g_top, _ = scattered_field_pwe(lam, particles, coefs, ls, i_top, kappa, alpha)
    _, g_bot = scattered_field_pwe(lam, particles, coefs, ls, 0, kappa, alpha)
    _, init_bot = initial_field.plane_wave_expansion(ls, 0)
    init_top, _ = initial_field.plane_wave_expansion(ls, i_top)
    kz_bot = k_z(kappa, k_bot)
    kz_top = k_z(kappa, k_top)
    p_bot = 4 * np.pi ** 2 * kz_bot / omega * (init_bot['g'][pol_P] * np.conj(g_bot[pol_P, 0, 0])).real
    p_top = 4 * np.pi ** 2 * kz_top / omega * (init_top['g'][pol_P] * np.conj(g_top[pol_P, 0, 0])).real
    return float(np.real(-p_bot / I0) + np.real(-p_top / I0))


def total_scattering_cross_section(initial_field, particles, coefs, ls, angular_resolution=np.pi / 360):
    """far_field.py:480-514 via scattered_far_field (:363-427) and pwe_to_ff_conversion (:217-254)."""
    lam = initial_field.vacuum_wavelength
    omega = angular_frequency(lam)
    az, po = angular_arrays(angular_resolution)
    i_top = ls.number_of_layers() - 1
    beta = initial_field.polar_angle
    i_P = 0 if np.cos(beta) > 0 else i_top
    n_P = np.real(ls.refractive_indices[i_P])
    I0 = abs(initial_field.amplitude) ** 2 * n_P / 2
    parts = []
    top = po[po < np.pi / 2]
    bot = po[po > np.pi / 2]
    for layer, sel, kind in ((i_top, top, 'upgoing'), (0, bot, 'downgoing')):
        n_l = ls.refractive_indices[layer]
        if len(sel) <= 1 or np.imag(n_l) != 0:
            continue
        neff = np.sort(np.sin(sel) * n_l)
        kp = neff * omega
        gu, gd = scattered_field_pwe(lam, particles, coefs, ls, layer, kp, az)
        g = gu if kind == 'upgoing' else gd
        k = omega * n_l
        polar = np.arcsin(kp / k) if kind == 'upgoing' else np.pi - np.arcsin(kp / k)
        kz = k_z(kp, k)
        intens = (2 * np.pi ** 2 / omega * (kz ** 2 * k)[None, :, None] * abs(g) ** 2).real
        srt = np.argsort(polar)
        parts.append((np.real(polar[srt]), intens[:, srt, :]))
    parts.sort(key=lambda t: t[0][0])
    polar = np.concatenate([p[0] for p in parts])
    sig = np.concatenate([p[1] for p in parts], axis=1) / I0
    per_pol = np.trapezoid(np.trapezoid(sig, az[None, None, :]) * np.sin(polar[None, :]), polar[None, :])
    return float(per_pol[0] + per_pol[1])
