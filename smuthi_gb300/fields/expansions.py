"""Field expansions: spherical-wave coefficients and plane-wave expansions with GPU field evaluation.

Mirrors smuthi/fields/expansions.py: ``SphericalWaveExpansion`` (:242-463) as a coefficient
container, and ``PlaneWaveExpansion`` (:466-1000) whose electric and magnetic fields at points run on
the GPU through ``sg_pwe_field`` (FP64) where the reference runs its FP32 kernels
(smuthi/fields/expansions_cuda.py:5-421). A discrete expansion (a single in-plane wavenumber) is
evaluated on the host exactly as the reference does (its GPU branch needs more than one).
"""
import numpy as np

from . import angular_frequency, blocksize
from . import k_z as _k_z


class FieldExpansion:
    """Base class: validity conditions shared by all expansions (reference :22-92)."""

    def __init__(self):
        self.validity_conditions = []

    def valid(self, x, y, z):
        vld = np.ones(np.shape(x), dtype=bool)
        for check in self.validity_conditions:
            vld = np.logical_and(vld, check(x, y, z))
        return vld


class SphericalWaveExpansion(FieldExpansion):
    """Coefficients a_{tau l m} of a regular or outgoing SWE about a reference point."""

    def __init__(self, k, l_max, m_max=None, kind=None, reference_point=None, lower_z=-np.inf, upper_z=np.inf):
        FieldExpansion.__init__(self)
        self.k = k
        self.l_max = l_max
        self.m_max = l_max if m_max is None else m_max
        self.kind = kind
        self.reference_point = reference_point
        self.lower_z = lower_z
        self.upper_z = upper_z
        self.coefficients = np.zeros(blocksize(self.l_max, self.m_max), dtype=complex)

    def __add__(self, other):
        out = SphericalWaveExpansion(self.k, self.l_max, self.m_max, self.kind, self.reference_point,
                                     max(self.lower_z, other.lower_z), min(self.upper_z, other.upper_z))
        out.coefficients = self.coefficients + other.coefficients
        return out


_default_contexts = {}


def _context(context):
    """The caller's library context, else one default context per process (device 0)."""
    if context is not None:
        return context
    if 0 not in _default_contexts:
        from .._lib import Context
        _default_contexts[0] = Context(0)
    return _default_contexts[0]


class PlaneWaveExpansion(FieldExpansion):
    """E(r) = sum_j int d^2k_par g_j(kappa, alpha) Phi_j(kappa, alpha; r - r_ref) in [lower_z, upper_z).

    ``coefficients[j, k, a]`` = g_j(kappa_k, alpha_a), j = 0 (TE), 1 (TM); ``kind`` 'upgoing' or
    'downgoing' (the sign of k_z). Field evaluation: ``electric_field`` / ``magnetic_field``
    (reference :635-783); ``max_chunksize`` and ``cpu_precision`` are accepted for signature
    compatibility, the GPU evaluation is FP64. ``context``: the library context to run on (default:
    one per process on device 0).
    """

    def __init__(self, k, k_parallel, azimuthal_angles, kind=None, reference_point=None, lower_z=-np.inf,
                 upper_z=np.inf):
        FieldExpansion.__init__(self)
        self.k = k
        self.k_parallel = np.array(k_parallel, ndmin=1)
        self.azimuthal_angles = np.array(azimuthal_angles, ndmin=1)
        self.kind = kind
        self.reference_point = reference_point
        self.lower_z = lower_z
        self.upper_z = upper_z
        self.coefficients = np.zeros((2, len(self.k_parallel), len(self.azimuthal_angles)), dtype=complex)

    def set_reference_point(self, new_reference_point):
        """Move the reference point (phase factor on the coefficients, reference :524-547)."""
        kx = self.k_parallel_grid() * np.cos(self.azimuthal_angle_grid())
        ky = self.k_parallel_grid() * np.sin(self.azimuthal_angle_grid())
        d = np.array(new_reference_point) - np.array(self.reference_point)
        self.coefficients = self.coefficients * np.exp(1j * (kx * d[0] + ky * d[1] + self.k_z_grid() * d[2]))[None]
        self.reference_point = new_reference_point

    def valid(self, x, y, z):
        if self.upper_z == float('inf'):
            vld = np.asarray(z) >= self.lower_z
        else:
            vld = np.logical_and(np.asarray(z) >= self.lower_z, np.asarray(z) < self.upper_z)
        return np.logical_and(vld, FieldExpansion.valid(self, x, y, z))

    def diverging(self, x, y, z):
        return np.zeros(np.shape(x), dtype=bool)

    def k_parallel_grid(self):
        return np.meshgrid(self.k_parallel, self.azimuthal_angles, indexing='ij')[0]

    def azimuthal_angle_grid(self):
        return np.meshgrid(self.k_parallel, self.azimuthal_angles, indexing='ij')[1]

    def _sign(self):
        if self.kind == 'upgoing':
            return 1
        if self.kind == 'downgoing':
            return -1
        raise ValueError('pwe kind undefined')

    def k_z(self):
        return self._sign() * _k_z(k_parallel=self.k_parallel, k=self.k)

    def k_z_grid(self):
        return self._sign() * _k_z(k_parallel=self.k_parallel_grid(), k=self.k)

    def compatible(self, other):
        return (type(other).__name__ == "PlaneWaveExpansion" and np.isclose(self.k, other.k)
                and all(np.isclose(self.k_parallel, other.k_parallel))
                and all(np.isclose(self.azimuthal_angles, other.azimuthal_angles)) and self.kind == other.kind
                and np.array_equal(self.reference_point, other.reference_point))

    def __add__(self, other):
        if not self.compatible(other):
            raise ValueError('Plane wave expansion are inconsistent.')
        out = PlaneWaveExpansion(k=self.k, k_parallel=self.k_parallel, azimuthal_angles=self.azimuthal_angles,
                                 kind=self.kind, reference_point=self.reference_point,
                                 lower_z=max(self.lower_z, other.lower_z), upper_z=min(self.upper_z, other.upper_z))
        out.coefficients = self.coefficients + other.coefficients
        return out

    def _field(self, field, x, y, z, omega, context):
        x, y, z = (np.asarray(v, dtype=float) for v in (x, y, z))
        out = [np.zeros(x.shape, dtype=complex) for _ in range(3)]
        vld = self.valid(x, y, z)
        xr = x[vld] - self.reference_point[0]
        yr = y[vld] - self.reference_point[1]
        zr = z[vld] - self.reference_point[2]
        if not xr.size:
            return tuple(out)
        if len(self.k_parallel) == 1:  # discrete expansion: the reference's host formula
            kp, a = self.k_parallel[0], self.azimuthal_angles[0]
            kz = self.k_z()[0]
            g0, g1 = self.coefficients[0, 0, 0], self.coefficients[1, 0, 0]
            if field == 0:
                comp = (-np.sin(a) * g0 + np.cos(a) * kz / self.k * g1, np.cos(a) * g0 + np.sin(a) * kz / self.k * g1,
                        -kp / self.k * g1)
            else:
                comp = (-kz * np.cos(a) * g0 - np.sin(a) * self.k * g1, -kz * np.sin(a) * g0 + np.cos(a) * self.k * g1,
                        kp * g0)
            kr = xr * kp * np.cos(a) + yr * kp * np.sin(a) + zr * kz
            eikr = (np.cos(kr.real) + 1j * np.sin(kr.real)) * np.exp(-kr.imag)
            for c in range(3):
                out[c][vld] = comp[c] * eikr / omega
            return tuple(out)
        import torch
        ctx = _context(context)
        dev = torch.device("cuda", ctx.device)
        stream = torch.cuda.current_stream(dev).cuda_stream

        def d(a, dtype):
            return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).to(dev)

        xd, yd, zd = d(xr, np.float64), d(yr, np.float64), d(zr, np.float64)
        kp_d, kz_d = d(self.k_parallel, np.complex128), d(self.k_z(), np.complex128)
        al_d, g_d = d(self.azimuthal_angles, np.float64), d(self.coefficients, np.complex128)
        res = torch.empty((3, xr.size), dtype=torch.complex128, device=dev)
        ctx.pwe_field_dev(field, xr.size, xd.data_ptr(), yd.data_ptr(), zd.data_ptr(), len(self.k_parallel),
                          kp_d.data_ptr(), kz_d.data_ptr(), len(self.azimuthal_angles), al_d.data_ptr(),
                          g_d.data_ptr(), complex(self.k), omega, res.data_ptr(), stream=stream)
        res = res.cpu().numpy()
        for c in range(3):
            out[c][vld] = res[c]
        return tuple(out)

    def electric_field(self, x, y, z, max_chunksize=50, cpu_precision='single precision', context=None):
        """(E_x, E_y, E_z) at the points (zero outside the expansion's validity range)."""
        return self._field(0, x, y, z, 1.0, context)

    def magnetic_field(self, x, y, z, vacuum_wavelength, max_chunksize=50, cpu_precision='single precision',
                       context=None):
        """(H_x, H_y, H_z) at the points (zero outside the expansion's validity range)."""
        return self._field(1, x, y, z, angular_frequency(vacuum_wavelength), context)
