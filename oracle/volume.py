"""Oracle: volumetric (different-height) coupling lookup and its CPU matvec.

TEST INFRASTRUCTURE ONLY (see the package docstring). Restates

* ``volumetric_coupling_lookup_table``
  (smuthi/linearsystem/particlecoupling/prepare_lookup.py:16-250): the 2-D tables
  w_pl[rho, z1 + z2, n1, n2] (layer-mediated, "plus") and w_mn[rho, z1 - z2, n1, n2]
  (direct + layer-mediated, "minus"), held in complex64 like the reference (:79-84);
* ``CouplingMatrixVolumeLookupCPU`` (smuthi/linearsystem/linear_system.py:592-667):
  scipy ``RectBivariateSpline`` with kx = ky = 1 ('linear') or 3 ('cubic') on the
  (rho, z) grids and M = (M_pl(rho, z1 + z2) + M_mn(rho, z1 - z2)) e^{i (m2 - m1) phi};
* the 4 x 4-tap Catmull-Rom interpolation of ``CouplingMatrixVolumeLookupCUDA``'s cubic
  kernel (smuthi/linearsystem/linear_system_cuda.py:149-272), evaluated in float64
  ('cubic_hermite');
* the tensor-product not-a-knot cubic spline in second-derivative (moment) form, the
  representation the GPU kernel uses for 'cubic': ``spline_moments`` / ``moment_spline_eval``
  are checked against ``RectBivariateSpline(kx=ky=3)`` here so that the formula itself is
  pinned on the CPU.
"""
import numpy as np
import scipy.interpolate
import scipy.special

from . import layers as lay
from .solve import system_layout
from .special import (ab5_coefficients, angular_frequency, blocksize, index_triples, k_z, legendre_normalized,
                      multi_to_single_index, spherical_hankel, transformation_coefficients_vwf)


def volumetric_coupling_lookup_table(vacuum_wavelength, particle_list, ls, k_parallel, resolution):
    """prepare_lookup.py:16-250 -> (w_pl, w_mn, rho_grid, sz_grid, dz_grid), tables complex64."""
    l_max = max(p.l_max for p in particle_list)
    m_max = max(p.m_max for p in particle_list)
    bs = blocksize(l_max, m_max)
    pos = np.array([p.position for p in particle_list], dtype=float)
    rho_pp = np.sqrt((pos[:, None, 0] - pos[None, :, 0]) ** 2 + (pos[:, None, 1] - pos[None, :, 1]) ** 2)
    z = pos[:, 2]
    dz_min, dz_max = z.min() - z.max(), z.max() - z.min()
    sz_min, sz_max = 2 * z.min(), 2 * z.max()
    rho = np.arange(-3 * resolution, rho_pp.max() + 3 * resolution, resolution)
    sz = np.arange(sz_min - 3 * resolution, sz_max + 3 * resolution, resolution)
    dz = np.arange(dz_min - 3 * resolution, dz_max + 3 * resolution, resolution)
    assert len(sz) == len(dz)
    nr, nz = len(rho), len(dz)
    i_s = ls.layer_number(particle_list[0].position[2])
    k_is = ls.wavenumber(i_s, vacuum_wavelength)
    z_is = ls.reference_z(i_s)
    wr_pl = np.zeros((nr, nz, bs, bs), dtype=np.complex64)
    wr_mn = np.zeros((nr, nz, bs, bs), dtype=np.complex64)

    # direct part on the (rho, z1 - z2) grid (:86-134)
    w = np.zeros((nr, nz, bs, bs), dtype=np.complex64)
    r = np.sqrt(dz[None, :] ** 2 + rho[:, None] ** 2)
    r[r == 0] = 1e-20
    ct = dz[None, :] / r
    st = rho[:, None] / r
    leg, _, _ = legendre_normalized(ct, st, 2 * l_max)
    hank = [spherical_hankel(n, k_is * r) for n in range(2 * l_max + 1)]
    err = np.seterr(over='ignore')  # the r = 1e-20 cells overflow complex64; they are zeroed below (:133)
    for m1 in range(-m_max, m_max + 1):
        for m2 in range(-m_max, m_max + 1):
            for l1 in range(max(1, abs(m1)), l_max + 1):
                for l2 in range(max(1, abs(m2)), l_max + 1):
                    A = np.zeros((nr, nz), dtype=complex)
                    B = np.zeros((nr, nz), dtype=complex)
                    for ld in range(max(abs(l1 - l2), abs(m1 - m2)), l1 + l2 + 1):
                        a5, b5 = ab5_coefficients(l2, m2, l1, m1, ld)
                        A += a5 * hank[ld] * leg[ld, abs(m1 - m2)]
                        B += b5 * hank[ld] * leg[ld, abs(m1 - m2)]
                    for t1 in range(2):
                        n1 = multi_to_single_index(t1, l1, m1, l_max, m_max)
                        for t2 in range(2):
                            n2 = multi_to_single_index(t2, l2, m2, l_max, m_max)
                            w[:, :, n1, n2] = A if t1 == t2 else B
    np.seterr(**err)
    w[rho < rho_pp[~np.eye(len(particle_list), dtype=bool)].min() / 2, :, :, :] = 0

    if not ls.is_degenerate():
        # layer-mediated part (:137-248), trapezoidal rule of the host branch (:239-245)
        kp = np.asarray(k_parallel)
        kz = k_z(kp, k_is)
        epl_sz = np.exp(1j * kz[None, :] * (sz[:, None] - 2 * z_is))
        emn_sz = np.exp(-1j * kz[None, :] * (sz[:, None] - 2 * z_is))
        epl_dz = np.exp(1j * kz[None, :] * dz[:, None])
        emn_dz = np.exp(-1j * kz[None, :] * dz[:, None])
        omega = angular_frequency(vacuum_wavelength)
        L = np.zeros((2, 2, 2, len(kp)), complex)
        for pol in range(2):
            L[pol] = lay.response_matrix(pol, ls.thicknesses, ls.refractive_indices, kp, omega, i_s, i_s)
        Bd = np.zeros((2, 2, bs, len(kp)), complex)
        Bn = np.zeros((2, 2, bs, len(kp)), complex)
        _, pi_pl, tau_pl = legendre_normalized(kz / k_is, kp / k_is, l_max)
        _, pi_mn, tau_mn = legendre_normalized(-kz / k_is, kp / k_is, l_max)
        m_of = [None] * bs
        for tau in range(2):
            for m in range(-m_max, m_max + 1):
                for l in range(max(1, abs(m)), l_max + 1):
                    n = multi_to_single_index(tau, l, m, l_max, m_max)
                    m_of[n] = m
                    for pol in range(2):
                        Bd[pol, 0, n] = transformation_coefficients_vwf(tau, l, m, pol, pi_pl, tau_pl, dagger=True)
                        Bd[pol, 1, n] = transformation_coefficients_vwf(tau, l, m, pol, pi_mn, tau_mn, dagger=True)
                        Bn[pol, 0, n] = transformation_coefficients_vwf(tau, l, m, pol, pi_pl, tau_pl)
                        Bn[pol, 1, n] = transformation_coefficients_vwf(tau, l, m, pol, pi_mn, tau_mn)
        combos = [[] for _ in range(2 * m_max + 1)]
        for n1 in range(bs):
            for n2 in range(bs):
                combos[abs(m_of[n1] - m_of[n2])].append((n1, n2))
        dkp = np.diff(kp)
        for dm in range(2 * m_max + 1):
            besjac = scipy.special.jv(dm, kp[None, :] * rho[:, None]) * (kp / (kz * k_is))[None, :]
            for n1, n2 in combos[dm]:
                bpl = np.zeros((nz, len(kp)), dtype=complex)
                bmn = np.zeros((nz, len(kp)), dtype=complex)
                for pol in range(2):
                    bpl += ((L[pol, 0, 1] * Bd[pol, 0, n1] * Bn[pol, 1, n2])[None, :] * epl_sz
                            + (L[pol, 1, 0] * Bd[pol, 1, n1] * Bn[pol, 0, n2])[None, :] * emn_sz)
                    bmn += ((L[pol, 0, 0] * Bd[pol, 0, n1] * Bn[pol, 0, n2])[None, :] * epl_dz
                            + (L[pol, 1, 1] * Bd[pol, 1, n1] * Bn[pol, 1, n2])[None, :] * emn_dz)
                f = besjac[:, None, :] * bpl[None, :, :]
                wr_pl[:, :, n1, n2] = 2 * (1j) ** abs(m_of[n2] - m_of[n1]) * (
                    (f[:, :, :-1] + f[:, :, 1:]) * dkp[None, None, :]).sum(axis=-1)
                f = besjac[:, None, :] * bmn[None, :, :]
                wr_mn[:, :, n1, n2] = 2 * (1j) ** abs(m_of[n2] - m_of[n1]) * (
                    (f[:, :, :-1] + f[:, :, 1:]) * dkp[None, None, :]).sum(axis=-1)
    return wr_pl, w + wr_mn, rho, sz, dz


def _catmull_rom(w):
    """Tap weights of the reference CUDA kernel's cubic_interpolation (linear_system_cuda.py:158-162)."""
    return np.array([-w ** 3 + 2 * w ** 2 - w, 3 * w ** 3 - 5 * w ** 2 + 2, -3 * w ** 3 + 4 * w ** 2 + w,
                     w ** 3 - w ** 2]) / 2


def spline_moments(f, axis):
    """h^2 * second derivative at every node of the not-a-knot cubic spline along ``axis``.

    Uniform nodes: interior rows m_{k-1} + 4 m_k + m_{k+1} = 6 (f_{k+1} - 2 f_k + f_{k-1}); the
    not-a-knot conditions (continuous third derivative at the second and the second-to-last
    node) make m_1 and m_{n-2} explicit and m_0 = 2 m_1 - m_2, m_{n-1} = 2 m_{n-2} - m_{n-3}.
    """
    f = np.moveaxis(np.asarray(f), axis, 0)
    n = f.shape[0]
    d = 6 * (f[2:] - 2 * f[1:-1] + f[:-2])  # rows 1 .. n-2
    m = np.zeros_like(f, dtype=np.result_type(f, float))
    m[1] = d[0] / 6
    m[n - 2] = d[-1] / 6
    nin = n - 4
    if nin > 0:
        rhs = d[1:-1].copy()  # rows 2 .. n-3
        rhs[0] -= m[1]
        rhs[-1] -= m[n - 2]
        A = np.diag(np.full(nin, 4.0)) + np.diag(np.ones(nin - 1), 1) + np.diag(np.ones(nin - 1), -1)
        m[2:n - 2] = np.linalg.solve(A, rhs.reshape(nin, -1)).reshape(rhs.shape)
    m[0] = 2 * m[1] - m[2]
    m[n - 1] = 2 * m[n - 2] - m[n - 3]
    return np.moveaxis(m, 0, axis)


def _moment_weights(u):
    """(value, moment) weights of the two nodes of a cubic-spline interval at fraction u."""
    a = np.array([1 - u, u])
    c = np.array([((1 - u) ** 3 - (1 - u)) / 6, (u ** 3 - u) / 6])
    return a, c


def moment_spline_eval(f, mx, my, mxy, ia, u, ib, v):
    """Tensor-product spline at fraction (u, v) of cell (ia, ib) from values and node moments."""
    au, cu = _moment_weights(u)
    av, cv = _moment_weights(v)
    s = 0
    for a in range(2):
        for b in range(2):
            s = s + (au[a] * av[b] * f[ia + a, ib + b] + cu[a] * av[b] * mx[ia + a, ib + b]
                     + au[a] * cv[b] * my[ia + a, ib + b] + cu[a] * cv[b] * mxy[ia + a, ib + b])
    return s


class VolumeLookupCPU:
    """CouplingMatrixVolumeLookupCPU (linear_system.py:592-667), plus 'cubic_hermite'."""

    def __init__(self, particle_list, table_pl, table_mn, rho_grid, sz_grid, dz_grid, kind='linear'):
        pos = np.array([p.position for p in particle_list], dtype=float)
        self.rho = np.sqrt((pos[:, None, 0] - pos[None, :, 0]) ** 2 + (pos[:, None, 1] - pos[None, :, 1]) ** 2)
        self.phi = np.arctan2(pos[:, None, 1] - pos[None, :, 1], pos[:, None, 0] - pos[None, :, 0])
        self.sz = pos[:, None, 2] + pos[None, :, 2]
        self.dz = pos[:, None, 2] - pos[None, :, 2]
        self.part, self.nlook, self.m, self.offs = system_layout(particle_list)
        self.bs = table_pl.shape[2]
        self.shape = (len(self.part), len(self.part))
        self.kind = kind
        self.grids = (rho_grid, sz_grid, dz_grid)
        self.tables = (np.asarray(table_pl), np.asarray(table_mn))
        self.sel = [np.where(self.nlook == n)[0] for n in range(self.bs)]
        self.m_of = np.zeros(self.bs, int)
        for n in range(self.bs):
            if len(self.sel[n]):
                self.m_of[n] = self.m[self.sel[n][0]]
        if kind in ('linear', 'cubic'):
            k = 1 if kind == 'linear' else 3
            sp = scipy.interpolate.RectBivariateSpline
            self.spl = [[[sp(rho_grid, g, t[:, :, a, b].real, kx=k, ky=k), sp(rho_grid, g, t[:, :, a, b].imag, kx=k,
                                                                              ky=k)]
                         for a in range(self.bs) for b in range(self.bs)]
                        for t, g in ((table_pl, sz_grid), (table_mn, dz_grid))]
        elif kind != 'cubic_hermite':
            raise ValueError(kind)

    def _hermite(self, t, grid, rho, zz, a, b):
        rg = self.grids[0]
        res = rg[1] - rg[0]
        out = np.zeros(rho.shape, complex)
        for idx in np.ndindex(rho.shape):
            ur = (rho[idx] - rg[0]) / res
            uz = (zz[idx] - grid[0]) / res
            ir, iz = int(np.floor(ur)), int(np.floor(uz))
            wr, wz = _catmull_rom(ur - np.floor(ur)), _catmull_rom(uz - np.floor(uz))
            blk = t[ir - 1:ir + 3, iz - 1:iz + 3, a, b].astype(complex)
            out[idx] = wr @ blk @ wz
        return out

    def element_block(self, n1, n2, i1, i2):
        """M[n1, n2] for receiver particles i1 (column) and emitters i2 (row), as a 2-D array."""
        rho = self.rho[i1[:, None], i2[None, :]]
        phi = self.phi[i1[:, None], i2[None, :]]
        sz = self.sz[i1[:, None], i2[None, :]]
        dz = self.dz[i1[:, None], i2[None, :]]
        if self.kind == 'cubic_hermite':
            mpl = self._hermite(self.tables[0], self.grids[1], rho, sz, n1, n2)
            mmn = self._hermite(self.tables[1], self.grids[2], rho, dz, n1, n2)
        else:
            e = n1 * self.bs + n2
            pr, pi = self.spl[0][e]
            mr, mi = self.spl[1][e]
            mpl = pr.ev(rho, sz) + 1j * pi.ev(rho, sz)
            mmn = mr.ev(rho, dz) + 1j * mi.ev(rho, dz)
        return (mpl + mmn) * np.exp(1j * (self.m_of[n2] - self.m_of[n1]) * phi)

    def matvec(self, x):
        x = np.asarray(x)
        out = np.zeros(x.shape, complex)
        for n1 in range(self.bs):
            idx1 = self.sel[n1]
            if not len(idx1):
                continue
            for n2 in range(self.bs):
                idx2 = self.sel[n2]
                if not len(idx2):
                    continue
                M = self.element_block(n1, n2, self.part[idx1], self.part[idx2])
                out[idx1] += M.dot(x[idx2])
        return out
