"""Extinction and total scattering cross sections of plane-wave excitations.

Mirrors ``extinction_cross_section`` (smuthi/postprocessing/far_field.py:517-654,
extinction_direction='both') and ``total_scattering_cross_section`` (:480-514,
via scattered_far_field :363-427 and pwe_to_ff_conversion :217-254). The
reference converts every particle's outgoing SWE to a plane wave expansion and
applies the layer response per particle (scattered_field.py:80-150,
transformations.py:133-233). For particles in one layer the conversion is
linear in the particles' coefficients, so here the particle sum is a matrix
product (coefficients x angular factors x lateral phase, times a per-particle
height factor when the particles sit at different heights) taken before the
layer response, which is applied once. Particles with a smaller multipole
cut-off enter with zeros at the indices they lack.
"""
import numpy as np

from .. import fields as flds
from .. import layers as lay
from ..fields.transformations import transformation_coefficients_vwf
from ..utility.math import legendre_normalized


def _particle_data(particle_list, coefficients=None):
    """(xy, z, l_max, m_max, coefficients) of the particles.

    z is a scalar when all particles share one height, else the per-particle heights. The
    coefficients are in the index layout of the largest cut-off (l_max, m_max): [N, B] or, for
    particles of one cut-off, also [R, N, B]; with mixed cut-offs they come one array per particle
    (``coefficients`` given as a sequence, or the particles' scattered fields) and are embedded
    with zeros.
    """
    pos = np.array([p.position for p in particle_list], dtype=float)
    l_max = max(p.l_max for p in particle_list)
    m_max = max(p.m_max for p in particle_list)
    zs = pos[:, 2]
    z = float(zs[0]) if np.all(zs == zs[0]) else zs
    if coefficients is None:
        coefficients = [p.scattered_field.coefficients for p in particle_list]
    if all((p.l_max, p.m_max) == (l_max, m_max) for p in particle_list):
        return pos[:, :2], z, l_max, m_max, np.asarray(coefficients)
    out = np.zeros((len(particle_list), flds.blocksize(l_max, m_max)), complex)
    for i, (p, c) in enumerate(zip(particle_list, coefficients)):
        tau, ll, mm = flds.index_table(p.l_max, p.m_max)
        gidx = [flds.multi_to_single_index(t, l, m, l_max, m_max) for t, l, m in zip(tau, ll, mm)]
        out[i, gidx] = np.asarray(c).ravel()
    return pos[:, :2], z, l_max, m_max, out


def scattered_pwe(vacuum_wavelength, layer_system, xy, z, l_max, m_max, coefs, layer_number, kpar, alpha,
                  chunk=16, context=None, include_direct=True, include_layer_response=True):
    """(g_up, g_down) [nrhs, 2, K, A] of the scattered field in ``layer_number``.

    coefs: [nrhs, N, blocksize] outgoing SWE coefficients (or [N, blocksize]); z: the particles'
    common height, or one height per particle. With a library ``context`` (and real ``kpar``) the
    particle sum runs on that context's GPU (``sg_farfield_sum_heights``, FP64); the angular factors
    and the layer response stay on the host. ``include_direct`` / ``include_layer_response`` select
    the two parts as in the reference (scattered_field.py:125-148).
    """
    coefs = np.asarray(coefs)
    single = coefs.ndim == 2
    if single:
        coefs = coefs[None]
    R = coefs.shape[0]
    kpar = np.atleast_1d(np.asarray(kpar))
    alpha = np.atleast_1d(np.asarray(alpha, dtype=float))
    omega = flds.angular_frequency(vacuum_wavelength)
    heights = np.ndim(z) > 0
    i_s = layer_system.layer_number(z[0] if heights else z)
    k = omega * layer_system.refractive_indices[i_s]
    kz = flds.k_z(k_parallel=kpar, k=k)
    dz = layer_system.reference_z(i_s) - np.asarray(z)  # scalar, or [N] for particles at different heights
    tau, ll, mm = flds.index_table(l_max, m_max)
    nm = 2 * m_max + 1
    gs = []
    if context is not None:
        import torch
        if np.iscomplexobj(kpar) and np.any(np.imag(kpar) != 0):
            raise ValueError('the GPU far-field sum needs real in-plane wavenumbers')
        dev = torch.device("cuda", context.device)
        stream = torch.cuda.current_stream(dev).cuda_stream
        N = coefs.shape[1]
        c_d = torch.from_numpy(np.ascontiguousarray(np.transpose(coefs, (1, 2, 0)), dtype=np.complex128)).to(dev)
        xy_d = torch.from_numpy(np.ascontiguousarray(xy, dtype=np.float64)).to(dev)
        kp_d = torch.from_numpy(np.ascontiguousarray(np.real(kpar), dtype=np.float64)).to(dev)
        al_d = torch.from_numpy(np.ascontiguousarray(alpha, dtype=np.float64)).to(dev)
    for sgn in (1, -1):  # up, down
        _, pilm, taulm = legendre_normalized(sgn * kz / k, kpar / k, l_max)
        # S[n, pol, K, m]: angular coefficient, nonzero only for m == m(n)
        S = np.zeros((len(tau), 2, len(kpar), nm), complex)
        for n in range(len(tau)):
            for pol in range(2):
                S[n, pol, :, mm[n] + m_max] = transformation_coefficients_vwf(tau[n], ll[n], mm[n], pol, pilm, taulm)
        if heights:
            pref = 1 / (2 * np.pi * kz * k)
            zph = np.exp(1j * sgn * kz[:, None] * dz[None, :])  # [K, N]
        else:
            pref = np.exp(1j * sgn * kz * dz) / (2 * np.pi * kz * k)
            zph = None
        if context is not None:
            Sn = np.ascontiguousarray(S[np.arange(len(tau)), :, :, mm + m_max])  # [n, pol, K]
            S_d = torch.from_numpy(Sn).to(dev)
            zph_d = None if zph is None else torch.from_numpy(np.ascontiguousarray(zph)).to(dev)
            out = torch.empty((R, 2, len(kpar), len(alpha)), dtype=torch.complex128, device=dev)
            context.farfield_sum_dev(N, xy_d.data_ptr(), len(tau), R, c_d.data_ptr(), m_max, mm, len(kpar),
                                     kp_d.data_ptr(), S_d.data_ptr(), len(alpha), al_d.data_ptr(), out.data_ptr(),
                                     stream=stream, zphase_ptr=None if zph_d is None else zph_d.data_ptr())
            gs.append(out.cpu().numpy() * pref[None, None, :, None])
            continue
        D = np.einsum('rin,npkm->rpkmi', coefs, S)  # [R, 2, K, m, N]
        eima = np.exp(1j * np.outer(np.arange(-m_max, m_max + 1), alpha))  # [m, A]
        g = np.zeros((R, 2, len(kpar), len(alpha)), complex)
        for k0 in range(0, len(kpar), chunk):
            ks = slice(k0, k0 + chunk)
            kp = kpar[ks]
            ph = np.exp(-1j * kp[:, None, None] * (np.cos(alpha)[None, :, None] * xy[None, None, :, 0]
                                                   + np.sin(alpha)[None, :, None] * xy[None, None, :, 1]))
            if zph is not None:
                ph = ph * zph[ks][:, None, :]
            # sum over particles, then over m
            F = np.einsum('kai,rpkmi->rpkam', ph, D[:, :, ks])
            g[:, :, ks, :] = np.einsum('rpkam,ma->rpka', F, eima)
        gs.append(g * pref[None, None, :, None])
    g_up, g_dn = gs
    out_up = np.zeros_like(g_up)
    out_dn = np.zeros_like(g_dn)
    if i_s == layer_number and include_direct:
        out_up += g_up
        out_dn += g_dn
    for pol in range(2 if include_layer_response else 0):
        L = lay.layersystem_response_matrix(pol, layer_system.thicknesses, layer_system.refractive_indices, kpar,
                                            omega, i_s, layer_number)
        out_up[:, pol] += L[0, 0][None, :, None] * g_up[:, pol] + L[0, 1][None, :, None] * g_dn[:, pol]
        out_dn[:, pol] += L[1, 0][None, :, None] * g_up[:, pol] + L[1, 1][None, :, None] * g_dn[:, pol]
    if single:
        return out_up[0], out_dn[0]
    return out_up, out_dn


def _simulation_context(simulation, context):
    """The GPU context of a simulation's coupling matrix, when the caller gave none."""
    if context is not None or simulation is None:
        return context
    cm = getattr(getattr(simulation, 'linear_system', None), 'coupling_matrix', None)
    return getattr(cm, 'context', None)


def _incidence(initial_field, layer_system):
    i_top = layer_system.number_of_layers() - 1
    i_P = 0 if np.cos(initial_field.polar_angle) > 0 else i_top
    n_P = layer_system.refractive_indices[i_P]
    if np.imag(n_P):
        raise ValueError('plane wave from absorbing layer: cross section undefined')
    return i_P, float(np.real(n_P))


def extinction_cross_section(simulation=None, initial_field=None, particle_list=None, layer_system=None,
                             coefficients=None, context=None):
    """Extinction cross section (top plus bottom extinction) of a plane wave (``context``: GPU particle
    sum, see ``scattered_pwe``)."""
    context = _simulation_context(simulation, context)
    initial_field = initial_field or simulation.initial_field
    particle_list = particle_list or simulation.particle_list
    layer_system = layer_system or simulation.layer_system
    if type(initial_field).__name__ != 'PlaneWave':
        raise ValueError('Cross section only defined for plane wave excitation.')
    xy, z, l_max, m_max, coefs = _particle_data(particle_list, coefficients)
    i_top = layer_system.number_of_layers() - 1
    lam = initial_field.vacuum_wavelength
    omega = flds.angular_frequency(lam)
    k_bot = omega * layer_system.refractive_indices[0]
    k_top = omega * layer_system.refractive_indices[-1]
    pol_P = initial_field.polarization
    beta, alpha = initial_field.polar_angle, initial_field.azimuthal_angle
    i_P, n_P = _incidence(initial_field, layer_system)
    k_P = k_bot if i_P == 0 else k_top
    kappa = np.sin(beta) * k_P
    kvec = np.array([np.cos(alpha) * kappa, np.sin(alpha) * kappa, k_P * np.cos(beta)])
    rvec = np.array([0, 0, layer_system.reference_z(i_P)]) - np.array(initial_field.reference_point)
    A_P = initial_field.amplitude * np.exp(1j * np.dot(kvec, rvec))
    I0 = abs(A_P) ** 2 * n_P / 2
    g_top, _ = scattered_pwe(lam, layer_system, xy, z, l_max, m_max, coefs, i_top, kappa, alpha, context=context)
    _, g_bot = scattered_pwe(lam, layer_system, xy, z, l_max, m_max, coefs, 0, kappa, alpha, context=context)
    _, init_bot = initial_field.plane_wave_expansion(layer_system, 0)
    init_top, _ = initial_field.plane_wave_expansion(layer_system, i_top)
    kz_bot = flds.k_z(k_parallel=kappa, k=k_bot)
    kz_top = flds.k_z(k_parallel=kappa, k=k_top)
    p_bot = 4 * np.pi ** 2 * kz_bot / omega * (init_bot.coefficients[pol_P] * np.conj(g_bot[pol_P, 0, 0])).real
    p_top = 4 * np.pi ** 2 * kz_top / omega * (init_top.coefficients[pol_P] * np.conj(g_top[pol_P, 0, 0])).real
    return float(np.real(-p_bot / I0) + np.real(-p_top / I0))


def total_scattering_cross_section(simulation=None, initial_field=None, particle_list=None, layer_system=None,
                                   polar_angles='default', azimuthal_angles='default', angular_resolution=None,
                                   coefficients=None, context=None):
    """Angle-integrated scattering cross section (trapezoidal rule over the far-field grid;
    ``context``: GPU particle sum, see ``scattered_pwe``)."""
    context = _simulation_context(simulation, context)
    initial_field = initial_field or simulation.initial_field
    particle_list = particle_list or simulation.particle_list
    layer_system = layer_system or simulation.layer_system
    if angular_resolution is not None:
        az, po = flds.angular_arrays(angular_resolution)
    else:
        az = flds.default_azimuthal_angles if isinstance(azimuthal_angles, str) else azimuthal_angles
        po = flds.default_polar_angles if isinstance(polar_angles, str) else polar_angles
        if az is None or po is None:
            az, po = flds.angular_arrays()
    xy, z, l_max, m_max, coefs = _particle_data(particle_list, coefficients)
    lam = initial_field.vacuum_wavelength
    omega = flds.angular_frequency(lam)
    _, n_P = _incidence(initial_field, layer_system)
    I0 = abs(initial_field.amplitude) ** 2 * n_P / 2
    i_top = layer_system.number_of_layers() - 1
    parts = []
    for layer, sel, up in ((i_top, po[po < np.pi / 2], True), (0, po[po > np.pi / 2], False)):
        n_l = layer_system.refractive_indices[layer]
        if len(sel) <= 1 or np.imag(n_l) != 0:
            continue
        kp = np.sort(np.sin(sel) * n_l) * omega
        gu, gd = scattered_pwe(lam, layer_system, xy, z, l_max, m_max, coefs, layer, kp, az, context=context)
        g = gu if up else gd
        k = omega * n_l
        polar = np.arcsin(kp / k) if up else np.pi - np.arcsin(kp / k)
        kz = flds.k_z(k_parallel=kp, k=k)
        intens = (2 * np.pi ** 2 / omega * (kz ** 2 * k)[None, :, None] * abs(g) ** 2).real
        order = np.argsort(polar)
        parts.append((np.real(polar[order]), intens[:, order, :]))
    parts.sort(key=lambda p: p[0][0])
    polar = np.concatenate([p[0] for p in parts])
    sig = np.concatenate([p[1] for p in parts], axis=1) / I0
    per_pol = np.trapezoid(np.trapezoid(sig, az[None, None, :]) * np.sin(polar[None, :]), polar[None, :])
    return float(per_pol[0] + per_pol[1])
