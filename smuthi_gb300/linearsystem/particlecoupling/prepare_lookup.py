"""Coupling lookup tables: radial w[rho, n1, n2] (particles at one height) and volumetric
w_pl[rho, z1 + z2, n1, n2], w_mn[rho, z1 - z2, n1, n2] (particles at different heights).

The radial table follows smuthi/linearsystem/particlecoupling/prepare_lookup.py:253-464:

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

The volumetric tables follow prepare_lookup.py:16-250 (see ``volumetric_coupling_lookup_table``).
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

    With a library ``context`` the Bessel factors J_|dm|(kappa rho) * jac are evaluated on that
    context's GPU by ``sg_bessel_jac_table`` and stay there, and the contour sum with the per-(n1, n2)
    integrand runs on the same GPU in the library's own FP64 contraction kernel
    (``sg_lookup_contract``); only the small integrand (B^2 x len(kappa)) is formed on the host.
    Without a context both run on the host with scipy and numpy, as the reference does.
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
    dmat = np.abs(mm[:, None] - mm[None, :])
    if context is not None:
        return _layer_mediated_contract_device(kp, jac, rho, X, Bn, wts, dmat, m_max, bs, context)
    wr = np.zeros((len(rho), bs * bs), complex)
    for dm in range(2 * m_max + 1):
        n1s, n2s = np.nonzero(dmat == dm)
        if len(n1s) == 0:
            continue
        belbe = np.einsum('pcak,pcak->ak', X[:, :, n1s, :], Bn[:, :, n2s, :])  # [pairs, k]
        G = (belbe * wts[None, :]).T  # [k, pairs]
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


def volume_grids(positions, resolution):
    """(rho, sz, dz) grids of the volume lookup (prepare_lookup.py:57-73) and the smallest lateral
    particle distance."""
    pos = np.asarray(positions, dtype=float)
    dmax, dmin = pair_distance_extremes(pos[:, :2])
    z = pos[:, 2]
    rho = np.arange(-3 * resolution, dmax + 3 * resolution, resolution)
    sz = np.arange(2 * z.min() - 3 * resolution, 2 * z.max() + 3 * resolution, resolution)
    dz = np.arange(z.min() - z.max() - 3 * resolution, z.max() - z.min() + 3 * resolution, resolution)
    if len(sz) != len(dz):
        raise ValueError('volume lookup: z1 + z2 and z1 - z2 grids differ in length')
    return rho, sz, dz, dmin


def direct_part_volume(k_is, rho, dz, l_max, m_max, rho_min_pair):
    """Direct SVWF coupling on the (rho, z1 - z2) grid in complex64 [len_rho, len_dz, B, B].

    prepare_lookup.py:86-134: per (m1, m2, l1, l2) the sum over ld of a5/b5 * h_ld(k r) *
    P_ld^{|m1-m2|}(cos theta) with r = sqrt(rho^2 + dz^2) (r = 0 replaced by 1e-20), in the
    reference's order of operations and rounded once to complex64 like the reference array; zeroed
    below half the smallest lateral particle distance (:133).
    """
    bs = flds.blocksize(l_max, m_max)
    r = np.sqrt(dz[None, :] ** 2 + rho[:, None] ** 2)
    r[r == 0] = 1e-20
    leg, _, _ = legendre_normalized(dz[None, :] / r, rho[:, None] / r, 2 * l_max)
    hank = [spherical_hankel(n, k_is * r) for n in range(2 * l_max + 1)]
    w = np.zeros((len(rho), len(dz), bs, bs), dtype=np.complex64)
    with np.errstate(over='ignore'):  # r = 1e-20 rows overflow complex64; they are zeroed below
        for m1 in range(-m_max, m_max + 1):
            for m2 in range(-m_max, m_max + 1):
                dm = abs(m1 - m2)
                for l1 in range(max(1, abs(m1)), l_max + 1):
                    for l2 in range(max(1, abs(m2)), l_max + 1):
                        A = np.zeros(r.shape, complex)
                        B = np.zeros(r.shape, complex)
                        for ld in range(max(abs(l1 - l2), dm), l1 + l2 + 1):
                            a5, b5 = ab5_coefficients(l2, m2, l1, m1, ld)
                            A += a5 * hank[ld] * leg[ld, dm]
                            B += b5 * hank[ld] * leg[ld, dm]
                        same = [flds.multi_to_single_index(t, l1, m1, l_max, m_max) for t in range(2)]
                        other = [flds.multi_to_single_index(t, l2, m2, l_max, m_max) for t in range(2)]
                        for t1 in range(2):
                            for t2 in range(2):
                                w[:, :, same[t1], other[t2]] = A if t1 == t2 else B
    w[rho < rho_min_pair / 2] = 0
    return w


def layer_mediated_volume(vacuum_wavelength, layer_system, i_s, rho, sz, dz, k_parallel, l_max, m_max,
                          context=None, max_columns=1 << 21):
    """Layer-mediated volume tables (wr_pl, wr_mn), complex64 [len_rho, len_z, B, B].

    prepare_lookup.py:137-248: per (n1, n2) the trapezoidal Sommerfeld integral
    2 i^|dm| sum_k (f_k + f_{k+1}) dkappa_k of f = J_dm(kappa rho) kappa/(k_z k) * belbee(z, kappa),
    with belbee_pl built from the z1 + z2 phases and belbee_mn from the z1 - z2 phases. Here the
    trapezoid weights are folded into belbee and, per |dm|, every (z, n1, n2) column is one matrix
    product with the Bessel factors (evaluated on the context's GPU when one is given, as for the
    radial table); the result is rounded to complex64 like the reference arrays.
    """
    k_is = layer_system.wavenumber(i_s, vacuum_wavelength)
    z_is = layer_system.reference_z(i_s)
    omega = flds.angular_frequency(vacuum_wavelength)
    kp = np.asarray(k_parallel)
    kz = flds.k_z(k_parallel=kp, k=k_is)
    tau, ll, mm = flds.index_table(l_max, m_max)
    bs = len(tau)
    _, pi_pl, ta_pl = legendre_normalized(kz / k_is, kp / k_is, l_max)
    _, pi_mn, ta_mn = legendre_normalized(-kz / k_is, kp / k_is, l_max)
    Bd = np.zeros((2, 2, bs, len(kp)), complex)
    Bn = np.zeros((2, 2, bs, len(kp)), complex)
    L = np.zeros((2, 2, 2, len(kp)), complex)
    for pol in range(2):
        L[pol] = lay.layersystem_response_matrix(pol, layer_system.thicknesses, layer_system.refractive_indices, kp,
                                                 omega, i_s, i_s)
        for n in range(bs):
            Bd[pol, 0, n] = transformation_coefficients_vwf(tau[n], ll[n], mm[n], pol, pi_pl, ta_pl, dagger=True)
            Bd[pol, 1, n] = transformation_coefficients_vwf(tau[n], ll[n], mm[n], pol, pi_mn, ta_mn, dagger=True)
            Bn[pol, 0, n] = transformation_coefficients_vwf(tau[n], ll[n], mm[n], pol, pi_pl, ta_pl)
            Bn[pol, 1, n] = transformation_coefficients_vwf(tau[n], ll[n], mm[n], pol, pi_mn, ta_mn)
    epl_sz = np.exp(1j * kz[None, :] * (sz[:, None] - 2 * z_is))  # [z, k]
    emn_sz = np.exp(-1j * kz[None, :] * (sz[:, None] - 2 * z_is))
    epl_dz = np.exp(1j * kz[None, :] * dz[:, None])
    emn_dz = np.exp(-1j * kz[None, :] * dz[:, None])
    dkp = np.diff(kp)
    wts = np.zeros(len(kp), complex)
    wts[:-1] += dkp
    wts[1:] += dkp
    jac = kp / (kz * k_is)
    nr, nz = len(rho), len(sz)
    wr_pl = np.zeros((nr, nz, bs * bs), dtype=np.complex64)
    wr_mn = np.zeros((nr, nz, bs * bs), dtype=np.complex64)
    besjac_all = _bessel_factors(kp, jac, rho, 2 * m_max, context)
    dmat = np.abs(mm[:, None] - mm[None, :])
    for dm in range(2 * m_max + 1):
        n1s, n2s = np.nonzero(dmat == dm)
        if len(n1s) == 0:
            continue
        besjac = (besjac_all[dm] if besjac_all is not None
                  else scipy.special.jv(dm, kp[None, :] * rho[:, None]) * jac[None, :])
        step = max(1, max_columns // nz)
        for c0 in range(0, len(n1s), step):
            a, b = n1s[c0:c0 + step], n2s[c0:c0 + step]
            # per pair and kappa: coefficients of the four phase terms (prepare_lookup.py:222-229)
            c_pl_p = np.einsum('pak,pak->ak', L[:, 0, 1][:, None, :] * Bd[:, 0, a], Bn[:, 1, b])
            c_pl_m = np.einsum('pak,pak->ak', L[:, 1, 0][:, None, :] * Bd[:, 1, a], Bn[:, 0, b])
            c_mn_p = np.einsum('pak,pak->ak', L[:, 0, 0][:, None, :] * Bd[:, 0, a], Bn[:, 0, b])
            c_mn_m = np.einsum('pak,pak->ak', L[:, 1, 1][:, None, :] * Bd[:, 1, a], Bn[:, 1, b])
            cols = a * bs + b
            for out, cp, cm, ep, em in ((wr_pl, c_pl_p, c_pl_m, epl_sz, emn_sz),
                                        (wr_mn, c_mn_p, c_mn_m, epl_dz, emn_dz)):
                G = (cp[None, :, :] * ep[:, None, :] + cm[None, :, :] * em[:, None, :]) * wts[None, None, :]
                G = G.reshape(nz * len(a), len(kp)).T  # [k, (z, pair)]
                res = 2 * ipow(dm) * (besjac @ G)  # [rho, (z, pair)]
                out[:, :, cols] = res.reshape(nr, nz, len(a))
    return wr_pl.reshape(nr, nz, bs, bs), wr_mn.reshape(nr, nz, bs, bs)


def _layer_mediated_contract_device(kp, jac, rho, X, Bn, wts, dmat, m_max, bs, context):
    """Layer-mediated table [len_rho, B, B] with the Bessel factors and the contour sum on the GPU."""
    import torch
    dev = torch.device("cuda", context.device)
    stream = torch.cuda.current_stream(dev).cuda_stream
    besjac = _bessel_factors(kp, jac, rho, 2 * m_max, context, keep_on_device=True)
    nr, nk = len(rho), len(kp)
    out = torch.zeros((nr, bs * bs), dtype=torch.complex128, device=dev)
    keep = []  # the integrand uploads live until the stream has run the contractions
    for dm in range(2 * m_max + 1):
        n1s, n2s = np.nonzero(dmat == dm)
        if len(n1s) == 0:
            continue
        belbe = np.einsum('pcak,pcak->ak', X[:, :, n1s, :], Bn[:, :, n2s, :])  # [pairs, k]
        g = torch.from_numpy(np.ascontiguousarray((belbe * wts[None, :]).T)).to(dev)  # [k, pairs]
        cols = torch.from_numpy((n1s * bs + n2s).astype(np.int32)).to(dev)
        keep += [g, cols]
        context.lookup_contract_dev(besjac[dm].data_ptr(), nr, nk, g.data_ptr(), len(n1s), cols.data_ptr(),
                                    2 * ipow(dm), out.data_ptr(), bs * bs, stream=stream)
    return out.cpu().numpy().reshape(nr, bs, bs)


def _bessel_factors(kp, jac, rho, nmax, context, keep_on_device=False):
    """J_n(kappa rho) * jac for n = 0..nmax on the context's GPU ([n, rho, kappa]); None without one."""
    if context is None:
        return None
    import torch
    dev = torch.device("cuda", context.device)
    stream = torch.cuda.current_stream(dev).cuda_stream
    kp_d = torch.from_numpy(np.ascontiguousarray(kp, dtype=np.complex128)).to(dev)
    jac_d = torch.from_numpy(np.ascontiguousarray(jac, dtype=np.complex128)).to(dev)
    rho_d = torch.from_numpy(np.ascontiguousarray(rho, dtype=np.float64)).to(dev)
    out = torch.empty((nmax + 1, len(rho), len(kp)), dtype=torch.complex128, device=dev)
    context.bessel_jac_table_dev(kp_d.data_ptr(), jac_d.data_ptr(), len(kp), rho_d.data_ptr(), len(rho), nmax,
                                 out.data_ptr(), stream=stream)
    return out if keep_on_device else out.cpu().numpy()


def volumetric_coupling_lookup_table(vacuum_wavelength, particle_list, layer_system, k_parallel='default',
                                     resolution=None, context=None):
    """(w_pl, w_mn, rho_grid, sz_grid, dz_grid) for particles at different heights in one layer.

    prepare_lookup.py:16-250: w_pl[rho, z1 + z2, n1, n2] is the layer-mediated coupling indexed by
    the sum of the heights, w_mn[rho, z1 - z2, n1, n2] the direct plus layer-mediated coupling
    indexed by their difference; both complex64 like the reference. ``context``: a library context
    whose GPU evaluates the Bessel factors (None: host scipy).
    """
    if resolution is None:
        resolution = vacuum_wavelength / 100
        sys.stdout.write('Setting lookup resolution to %f\n' % resolution)
    l_max = max(p.l_max for p in particle_list)
    m_max = max(p.m_max for p in particle_list)
    pos = np.array([p.position for p in particle_list], dtype=float)
    rho, sz, dz, dmin = volume_grids(pos, resolution)
    i_s = layer_system.layer_number(pos[0, 2])
    k_is = layer_system.wavenumber(i_s, vacuum_wavelength)
    w = direct_part_volume(k_is, rho, dz, l_max, m_max, dmin)
    if layer_system.is_degenerate():
        return np.zeros_like(w), w, rho, sz, dz
    if isinstance(k_parallel, str) and k_parallel == 'default':
        k_parallel = flds.default_Sommerfeld_k_parallel_array
    if k_parallel is None:
        raise ValueError('no Sommerfeld contour: pass k_parallel or set the default contour')
    wr_pl, wr_mn = layer_mediated_volume(vacuum_wavelength, layer_system, i_s, rho, sz, dz, k_parallel, l_max, m_max,
                                         context=context)
    return wr_pl, w + wr_mn, rho, sz, dz
