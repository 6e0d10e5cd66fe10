"""Radial coupling lookup table w[rho, n1, n2] for particles at one height.

Follows smuthi/linearsystem/particlecoupling/prepare_lookup.py:253-464:

* radial grid ``arange(-3 r, rho_max + 3 r, r)`` (:291);
* direct part: sum over ld of a5/b5 (l2, m2, l1, m1, ld) * h_ld(k rho) * P_ld^{|m1-m2|}(0)
  (:300-338), held in complex64 exactly like the reference (:301) and zeroed
  below half the smallest particle distance (:339-340). The per-(m1, m2, l1, l2)
  accumulation keeps the reference's order of floating-point operations so the
  complex64 rounding lands on the same values;
* layer-mediated part (:343-459): the trapezoidal Sommerfeld integral
  2 i^|dm| sum_k (f_k + f_{k+1}) dkappa_k with f = J_dm(kappa rho) kappa/(k_z k) *
  belbe(kappa). Instead of one numpy reduction per (n1, n2) it is evaluated as
  one complex matrix product per |dm|: the trapezoid weights (dkappa_{k-1} +
  dkappa_k) are folded into the belbe columns;
* result ``w + wr`` (complex128).
"""
import sys

import numpy as np
import scipy.special

from ... import fields as flds
from ... import layers as lay
from ...fields.transformations import ab5_coefficients, ipow, transformation_coefficients_vwf
from ...utility.math import legendre_normalized, spherical_hankel


def pair_distance_extremes(particle_xy):
    """(largest, smallest nonzero-index) pair distance of lateral positions.

    The largest distance is attained between convex-hull vertices and the
    smallest between nearest neighbours, so neither needs the N x N matrix;
    both are evaluated with the same sqrt(dx^2 + dy^2) as a full matrix would.
    """
    xy = np.asarray(particle_xy, dtype=float)
    n = len(xy)
    if n < 2:
        return 0.0, np.inf
    if n <= 64:
        d = np.sqrt((xy[:, None, 0] - xy[None, :, 0]) ** 2 + (xy[:, None, 1] - xy[None, :, 1]) ** 2)
        return float(d.max()), float(d[~np.eye(n, dtype=bool)].min())
    from scipy.spatial import ConvexHull, cKDTree
    try:
        hull = xy[ConvexHull(xy).vertices]
    except Exception:  # degenerate (collinear) sets: fall back to all points
        hull = xy
    dmax = 0.0
    for s in range(0, len(hull), 1024):
        h = hull[s:s + 1024]
        d = np.sqrt((h[:, None, 0] - hull[None, :, 0]) ** 2 + (h[:, None, 1] - hull[None, :, 1]) ** 2)
        dmax = max(dmax, float(d.max()))
    _, idx = cKDTree(xy).query(xy, k=2)
    j = idx[:, 1]
    dmin = float(np.sqrt((xy[:, 0] - xy[j, 0]) ** 2 + (xy[:, 1] - xy[j, 1]) ** 2).min())
    return dmax, dmin


def radial_grid(particle_xy, resolution):
    """Radial grid arange(-3 r, rho_max + 3 r, r) and the smallest particle distance."""
    dmax, dmin = pair_distance_extremes(particle_xy)
    return np.arange(-3 * resolution, dmax + 3 * resolution, resolution), dmin


def direct_part(k_is, rho, l_max, m_max, rho_min_pair):
    """Direct SVWF coupling table in complex64 [len_rho, B, B]."""
    bs = flds.blocksize(l_max, m_max)
    w = np.zeros((len(rho), bs, bs), dtype=np.complex64)
    hank = []
    for n in range(2 * l_max + 1):
        h = spherical_hankel(n, k_is * rho)
        h[rho <= 0] = np.nan
        hank.append(h)
    leg0 = legendre_normalized(np.array([0.0]), np.array([1.0]), 2 * l_max)[0]
    for m1 in range(-m_max, m_max + 1):
        for m2 in range(-m_max, m_max + 1):
            dm = abs(m1 - m2)
            for l1 in range(max(1, abs(m1)), l_max + 1):
                for l2 in range(max(1, abs(m2)), l_max + 1):
                    A = np.zeros(len(rho), complex)
                    B = np.zeros(len(rho), complex)
                    for ld in range(max(abs(l1 - l2), dm), l1 + l2 + 1):
                        a5, b5 = ab5_coefficients(l2, m2, l1, m1, ld)
                        A = A + a5 * hank[ld] * leg0[ld, dm]
                        B = B + b5 * hank[ld] * leg0[ld, dm]
                    same = [flds.multi_to_single_index(t, l1, m1, l_max, m_max) for t in range(2)]
                    other = [flds.multi_to_single_index(t, l2, m2, l_max, m_max) for t in range(2)]
                    for t1 in range(2):
                        for t2 in range(2):
                            w[:, same[t1], other[t2]] = A if t1 == t2 else B
    w[rho < rho_min_pair / 2, :, :] = 0
    return w


def layer_mediated_part(vacuum_wavelength, layer_system, i_s, dz, rho, k_parallel, l_max, m_max, context=None):
    """Layer-mediated coupling table (complex128) [len_rho, B, B].

    With a library ``context`` the Bessel factors J_|dm|(kappa rho) * jac (the dominant cost of the
    build) are evaluated on that context's GPU by ``sg_bessel_jac_table``; without one on the host with
    scipy, as the reference does. The contraction with the per-(n1, n2) integrand is a small FP64 GEMM
    on the host in both cases (a library FP64 GEMM on the device may use reduced-precision emulation).
    """
    k_is = layer_system.wavenumber(i_s, vacuum_wavelength)
    omega = flds.angular_frequency(vacuum_wavelength)
    kp = np.asarray(k_parallel)
    kz = flds.k_z(k_parallel=kp, k=k_is)
    epl = np.exp(2j * kz * dz)
    emn = np.exp(-2j * kz * dz)
    tau, ll, mm = flds.index_table(l_max, m_max)
    bs = len(tau)
    _, pi_pl, ta_pl = legendre_normalized(kz / k_is, kp / k_is, l_max)
    _, pi_mn, ta_mn = legendre_normalized(-kz / k_is, kp / k_is, l_max)
    # X[pol, c, n1, k] combines the response and the dagger coefficients of the receiving wave;
    # belbe[n1, n2, k] = sum_{pol, c} X[pol, c, n1, k] * B[pol, c, n2, k]
    X = np.zeros((2, 2, bs, len(kp)), complex)
    Bn = np.zeros((2, 2, bs, len(kp)), complex)
    for pol in range(2):
        L = lay.layersystem_response_matrix(pol, layer_system.thicknesses, layer_system.refractive_indices, kp,
                                            omega, i_s, i_s)
        for n in range(bs):
            bd_pl = transformation_coefficients_vwf(tau[n], ll[n], mm[n], pol, pi_pl, ta_pl, dagger=True)
            bd_mn = transformation_coefficients_vwf(tau[n], ll[n], mm[n], pol, pi_mn, ta_mn, dagger=True)
            Bn[pol, 0, n] = transformation_coefficients_vwf(tau[n], ll[n], mm[n], pol, pi_pl, ta_pl)
            Bn[pol, 1, n] = transformation_coefficients_vwf(tau[n], ll[n], mm[n], pol, pi_mn, ta_mn)
            X[pol, 0, n] = L[0, 0] * bd_pl + L[1, 0] * bd_mn * emn
            X[pol, 1, n] = L[0, 1] * bd_pl * epl + L[1, 1] * bd_mn
    dkp = np.diff(kp)
    wts = np.zeros(len(kp), complex)
    wts[:-1] += dkp
    wts[1:] += dkp
    jac = kp / (kz * k_is)
    wr = np.zeros((len(rho), bs * bs), complex)
    dmat = np.abs(mm[:, None] - mm[None, :])
    besjac_host = None
    if context is not None:
        import torch
        dev = torch.device("cuda", context.device)
        stream = torch.cuda.current_stream(dev).cuda_stream
        kp_d = torch.from_numpy(np.ascontiguousarray(kp, dtype=np.complex128)).to(dev)
        jac_d = torch.from_numpy(np.ascontiguousarray(jac, dtype=np.complex128)).to(dev)
        rho_d = torch.from_numpy(np.ascontiguousarray(rho, dtype=np.float64)).to(dev)
        besjac_dev = torch.empty((2 * m_max + 1, len(rho), len(kp)), dtype=torch.complex128, device=dev)
        context.bessel_jac_table_dev(kp_d.data_ptr(), jac_d.data_ptr(), len(kp), rho_d.data_ptr(), len(rho),
                                     2 * m_max, besjac_dev.data_ptr(), stream=stream)
        besjac_host = besjac_dev.cpu().numpy()
        del besjac_dev, kp_d, jac_d, rho_d
    for dm in range(2 * m_max + 1):
        n1s, n2s = np.nonzero(dmat == dm)
        if len(n1s) == 0:
            continue
        belbe = np.einsum('pcak,pcak->ak', X[:, :, n1s, :], Bn[:, :, n2s, :])  # [pairs, k]
        G = (belbe * wts[None, :]).T  # [k, pairs]
        if besjac_host is not None:
            wr[:, n1s * bs + n2s] = 2 * ipow(dm) * (besjac_host[dm] @ G)
        else:
            besjac = scipy.special.jv(dm, kp[None, :] * rho[:, None]) * jac[None, :]
            wr[:, n1s * bs + n2s] = 2 * ipow(dm) * (besjac @ G)
    return wr.reshape(len(rho), bs, bs)


def radial_coupling_lookup_table(vacuum_wavelength, particle_list, layer_system, k_parallel='default',
                                 resolution=None, context=None):
    """Return (lookup_table[rho, n1, n2], rho_grid) for particles at a common height.

    ``context``: a library context whose GPU evaluates the Bessel factors of the layer-mediated part
    (None: host scipy, the reference's arithmetic).
    """
    if resolution is None:
        resolution = vacuum_wavelength / 100
        sys.stdout.write('Setting lookup resolution to %f\n' % resolution)
    l_max = max(p.l_max for p in particle_list)
    m_max = max(p.m_max for p in particle_list)
    xy = np.array([p.position[:2] for p in particle_list], dtype=float)
    rho, dmin = radial_grid(xy, resolution)
    z = particle_list[0].position[2]
    i_s = layer_system.layer_number(z)
    k_is = layer_system.wavenumber(i_s, vacuum_wavelength)
    dz = z - layer_system.reference_z(i_s)
    w = direct_part(k_is, rho, l_max, m_max, dmin)
    if layer_system.is_degenerate():
        return w, rho
    if isinstance(k_parallel, str) and k_parallel == 'default':
        k_parallel = flds.default_Sommerfeld_k_parallel_array
    if k_parallel is None:
        raise ValueError('no Sommerfeld contour: pass k_parallel or set the default contour')
    wr = layer_mediated_part(vacuum_wavelength, layer_system, i_s, dz, rho, k_parallel, l_max, m_max,
                             context=context)
    return w + wr, rho
