"""Oracle: electric and magnetic field of a plane-wave expansion at points.

TEST INFRASTRUCTURE ONLY (see the package docstring). Restates the CPU branch of
``PlaneWaveExpansion.electric_field`` / ``magnetic_field`` with cpu_precision='double precision'
(smuthi/fields/expansions.py:635-900 and smuthi/utility/numba_helpers.py:8-160):

* points outside [lower_z, upper_z) give zero (``valid``, :549-566);
* coordinates relative to the reference point; k.r = x kx + y ky + z kz on the (kappa, alpha) grid,
  kz = +-sqrt(k^2 - kappa^2) (upgoing / downgoing, :592-608);
* e^{i k.r} evaluated as (cos Re + i sin Re) * exp(-Im) (numba_helpers.py:24-35);
* integrands (:882-904): E: TE (-sin a, cos a, 0) g_TE, TM (cos a kz/k, sin a kz/k, -kappa/k) g_TM;
  H: TE (-kz cos a, -kz sin a, kappa) g_TE, TM (-k sin a, k cos a, 0) g_TM;
* trapezoid over alpha with the (x_{k+1} - x_k) (y_{k+1} + y_k) / 2 sum (numba_helpers.py:8-16),
  times kappa, then numpy's trapezoid over the complex kappa contour; H carries 1 / omega.
"""
import numpy as np

from .special import angular_frequency, k_z


class PlaneWaveExpansion:
    """Data of smuthi.fields.expansions.PlaneWaveExpansion (:466-522)."""

    def __init__(self, k, k_parallel, azimuthal_angles, kind, reference_point, lower_z=-np.inf, upper_z=np.inf):
        self.k = k
        self.k_parallel = np.array(k_parallel, ndmin=1)
        self.azimuthal_angles = np.array(azimuthal_angles, ndmin=1)
        self.kind = kind
        self.reference_point = reference_point
        self.lower_z = lower_z
        self.upper_z = upper_z
        self.coefficients = np.zeros((2, len(self.k_parallel), len(self.azimuthal_angles)), dtype=complex)

    def valid(self, x, y, z):
        if self.upper_z == float('inf'):
            return z >= self.lower_z
        return np.logical_and(z >= self.lower_z, z < self.upper_z)

    def k_z(self):
        kz = k_z(self.k_parallel, self.k)
        return kz if self.kind == 'upgoing' else -kz

    def _integrands(self, field):
        kp = self.k_parallel[:, None]
        a = self.azimuthal_angles[None, :]
        kz = self.k_z()[:, None]
        g0, g1 = self.coefficients
        if field == 'E':
            ix = -np.sin(a) * g0 + np.cos(a) * kz / self.k * g1
            iy = np.cos(a) * g0 + np.sin(a) * kz / self.k * g1
            iz = -kp / self.k * g1
        else:
            ix = -kz * np.cos(a) * g0 - np.sin(a) * self.k * g1
            iy = -kz * np.sin(a) * g0 + np.cos(a) * self.k * g1
            iz = kp * g0 + 0 * g1
        return ix, iy, iz

    def field(self, x, y, z, field='E', vacuum_wavelength=None):
        x, y, z = (np.asarray(v, dtype=float) for v in (x, y, z))
        out = [np.zeros(x.shape, complex) for _ in range(3)]
        vld = self.valid(x, y, z)
        xr = x[vld] - self.reference_point[0]
        yr = y[vld] - self.reference_point[1]
        zr = z[vld] - self.reference_point[2]
        omega = 1.0 if field == 'E' else angular_frequency(vacuum_wavelength)
        kp = self.k_parallel[:, None]
        a = self.azimuthal_angles[None, :]
        kx, ky, kz = kp * np.cos(a), kp * np.sin(a), self.k_z()[:, None] + 0 * a
        kr = xr[:, None, None] * kx + yr[:, None, None] * ky + zr[:, None, None] * kz
        eikr = (np.cos(kr.real) + 1j * np.sin(kr.real)) * np.exp(-kr.imag)
        da = np.diff(self.azimuthal_angles)
        for c, integ in enumerate(self._integrands(field)):
            f = integ[None] * eikr  # [point, kappa, alpha]
            if len(self.k_parallel) > 1:
                ia = ((f[:, :, 1:] + f[:, :, :-1]) * da / 2.0).sum(axis=-1)
                out[c][vld] = 1 / omega * np.trapezoid(ia * self.k_parallel, self.k_parallel, axis=-1)
            else:
                out[c][vld] = 1 / omega * np.squeeze(f, axis=(1, 2))
        return tuple(out)
