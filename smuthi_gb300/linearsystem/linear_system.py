"""Linear system (1 - T W) b = T a on the GPU, mirroring smuthi/linearsystem/linear_system.py.

``CouplingMatrixRadialLookupCUDA`` is the drop-in for the reference class of
the same name (:813-900): same constructor, a ``SystemMatrix`` with
``shape``/``index_block``/``index`` and a scipy ``LinearOperator`` whose
``matvec`` runs the sm_103a coupling kernel. ``MasterMatrix`` fuses
``v - T W v`` into one device operator when the coupling matrix is the GPU
lookup, and ``LinearSystem.solve`` runs GMRES on the device through the C ABI
(``sg_gmres_solve``) with the reference's call semantics (:271-286).

``CouplingMatrixVolumeLookupCUDA`` is the drop-in for the reference class of the
same name (:686-783) for particles at different heights in one layer: 2-D
(rho, z1 +- z2) tables, interpolated by the sm_103a volume kernel.

Only the lookup paths exist here: particles in one layer,
``store_coupling_matrix=False`` and a lookup resolution. Every other branch of
the reference (explicit coupling, LU, periodic lattices) raises
``NotImplementedError``; nothing falls back to a CPU implementation.
"""
import sys
import time
import warnings

import numpy as np
import scipy.sparse.linalg

from .. import fields as flds
from .._lib import SG_FP32, SG_FP64, Context
from ..fields.expansions import SphericalWaveExpansion
from ..utility import cuda as cu
from .particlecoupling import prepare_lookup as look

PRECISIONS = {'fp64': SG_FP64, 'mixed': SG_FP32}


class SystemMatrix:
    """Operator on system vectors: particle-major blocks of (tau, l, m) coefficients."""

    def __init__(self, particle_list):
        self.particle_list = particle_list
        sizes = np.array([flds.blocksize(p.l_max, p.m_max) for p in particle_list], dtype=np.int64)
        self._offsets = np.concatenate([[0], np.cumsum(sizes)])
        self.shape = (int(self._offsets[-1]), int(self._offsets[-1]))

    def index_block(self, i):
        return range(int(self._offsets[i]), int(self._offsets[i + 1]))

    def index(self, i, tau, l, m):
        p = self.particle_list[i]
        return int(self._offsets[i]) + flds.multi_to_single_index(tau, l, m, p.l_max, p.m_max)


def unknown_layout(particle_list):
    """Per-unknown particle index, global lookup index and the m of every lookup index."""
    l_max = max(p.l_max for p in particle_list)
    m_max = max(p.m_max for p in particle_list)
    _, _, m_of_n = flds.index_table(l_max, m_max)
    part = []
    nlook = []
    cache = {}
    for i, p in enumerate(particle_list):
        key = (p.l_max, p.m_max)
        if key not in cache:
            tau, ll, mm = flds.index_table(p.l_max, p.m_max)
            cache[key] = np.array([flds.multi_to_single_index(t, l, m, l_max, m_max)
                                   for t, l, m in zip(tau, ll, mm)], dtype=np.int32)
        part.append(np.full(len(cache[key]), i, dtype=np.int32))
        nlook.append(cache[key])
    return np.concatenate(part), np.concatenate(nlook), m_of_n.astype(np.int32), l_max, m_max


class CouplingMatrixRadialLookup(SystemMatrix):
    """Builds the radial lookup table (host FP64) for particles at one height."""

    def __init__(self, vacuum_wavelength, particle_list, layer_system, k_parallel='default', resolution=None,
                 table_context=None):
        z = [p.position[2] for p in particle_list]
        if not all(zz == z[0] for zz in z):
            raise ValueError('radial lookup needs all particles at the same height')
        SystemMatrix.__init__(self, particle_list)
        self.l_max = max(p.l_max for p in particle_list)
        self.m_max = max(p.m_max for p in particle_list)
        self.blocksize = flds.blocksize(self.l_max, self.m_max)
        self.resolution = resolution
        self.lookup_table, self.radial_distance_array = look.radial_coupling_lookup_table(
            vacuum_wavelength=vacuum_wavelength, particle_list=particle_list, layer_system=layer_system,
            k_parallel=k_parallel, resolution=resolution, context=table_context)


class CouplingMatrixRadialLookupCUDA(CouplingMatrixRadialLookup):
    """GPU radial-lookup coupling matrix W (drop-in for the reference CUDA class).

    ``interpolator_kind``: 'linear' (scipy linear), 'cubic' (scipy's not-a-knot
    cubic spline, the CPU reference's meaning) or 'cubic_hermite' (the 4-tap
    formula of the reference CUDA kernel). ``cuda_blocksize`` is accepted for
    signature compatibility; launch shapes are chosen by the library.
    """

    def __init__(self, vacuum_wavelength, particle_list, layer_system, k_parallel='default', resolution=None,
                 cuda_blocksize=None, interpolator_kind='linear', device=0, context=None):
        if interpolator_kind not in ('linear', 'cubic', 'cubic_hermite'):
            raise ValueError('unknown interpolator_kind %r' % interpolator_kind)
        self.context = context if context is not None else Context(device)
        # the table's Bessel factors are evaluated on the same GPU
        CouplingMatrixRadialLookup.__init__(self, vacuum_wavelength, particle_list, layer_system, k_parallel,
                                            resolution, table_context=self.context)
        self.interpolator_kind = interpolator_kind
        self.unknown_particle, self.unknown_n, self.m_of_n, _, _ = unknown_layout(particle_list)
        xy = np.array([p.position[:2] for p in particle_list], dtype=np.float64)
        self.context.set_particles(xy, self.unknown_particle, self.unknown_n, self.blocksize, self.m_of_n)
        self.context.set_lookup(interpolator_kind, self.lookup_table, self.radial_distance_array[0],
                                self.resolution if self.resolution is not None else
                                self.radial_distance_array[1] - self.radial_distance_array[0])
        self.precision = SG_FP64

        def matvec(v):
            return self.context.coupling_matvec(np.asarray(v, dtype=complex).ravel(), self.precision)

        self.linear_operator = scipy.sparse.linalg.LinearOperator(shape=self.shape, matvec=matvec, dtype=complex)


class CouplingMatrixVolumeLookup(SystemMatrix):
    """Builds the volumetric lookup tables (reference :563-589) for particles in one layer."""

    def __init__(self, vacuum_wavelength, particle_list, layer_system, k_parallel='default', resolution=None,
                 table_context=None):
        layers_ = {layer_system.layer_number(p.position[2]) for p in particle_list}
        if len(layers_) != 1:
            raise ValueError('the volume lookup needs all particles in one layer')
        SystemMatrix.__init__(self, particle_list)
        self.l_max = max(p.l_max for p in particle_list)
        self.m_max = max(p.m_max for p in particle_list)
        self.blocksize = flds.blocksize(self.l_max, self.m_max)
        self.resolution = resolution
        lkup = look.volumetric_coupling_lookup_table(vacuum_wavelength=vacuum_wavelength, particle_list=particle_list,
                                                     layer_system=layer_system, k_parallel=k_parallel,
                                                     resolution=resolution, context=table_context)
        self.lookup_table_plus, self.lookup_table_minus = lkup[0], lkup[1]
        self.rho_array, self.sum_z_array, self.diff_z_array = lkup[2], lkup[3], lkup[4]


class CouplingMatrixVolumeLookupCUDA(CouplingMatrixVolumeLookup):
    """GPU volume-lookup coupling matrix W (drop-in for the reference CUDA class, :686-783).

    ``interpolator_kind``: 'linear' (bilinear; the CPU and the CUDA reference agree), 'cubic'
    (tensor-product not-a-knot spline, the CPU reference's RectBivariateSpline meaning) or
    'cubic_hermite' (the 4 x 4-tap formula of the reference CUDA kernel). ``cuda_blocksize`` is
    accepted for signature compatibility.
    """

    def __init__(self, vacuum_wavelength, particle_list, layer_system, k_parallel='default', resolution=None,
                 cuda_blocksize=None, interpolator_kind='linear', device=0, context=None):
        if interpolator_kind not in ('linear', 'cubic', 'cubic_hermite'):
            raise ValueError('unknown interpolator_kind %r' % interpolator_kind)
        self.context = context if context is not None else Context(device)
        CouplingMatrixVolumeLookup.__init__(self, vacuum_wavelength, particle_list, layer_system, k_parallel,
                                            resolution, table_context=self.context)
        self.interpolator_kind = interpolator_kind
        self.unknown_particle, self.unknown_n, self.m_of_n, _, _ = unknown_layout(particle_list)
        pos = np.array([p.position for p in particle_list], dtype=np.float64)
        self.context.set_particles(pos[:, :2], self.unknown_particle, self.unknown_n, self.blocksize, self.m_of_n)
        res = self.rho_array[1] - self.rho_array[0] if self.resolution is None else self.resolution
        self.context.set_volume_lookup(interpolator_kind, pos[:, 2], self.lookup_table_plus, self.lookup_table_minus,
                                       self.rho_array[0], self.sum_z_array[0], self.diff_z_array[0], res)
        self.precision = SG_FP64

        def matvec(v):
            return self.context.coupling_matvec(np.asarray(v, dtype=complex).ravel(), self.precision)

        self.linear_operator = scipy.sparse.linalg.LinearOperator(shape=self.shape, matvec=matvec, dtype=complex)


GPU_COUPLING_MATRICES = (CouplingMatrixRadialLookupCUDA, CouplingMatrixVolumeLookupCUDA)


class TMatrix(SystemMatrix):
    """Block-diagonal system T-matrix (reference :410-438)."""

    def __init__(self, particle_list):
        SystemMatrix.__init__(self, particle_list)

        def apply_t_matrix(vector):
            out = np.zeros(vector.shape, dtype=complex)
            for i, p in enumerate(particle_list):
                sl = slice(int(self._offsets[i]), int(self._offsets[i + 1]))
                out[sl] = p.t_matrix.dot(vector[sl])
            return out

        self.linear_operator = scipy.sparse.linalg.LinearOperator(shape=self.shape, matvec=apply_t_matrix,
                                                                  matmat=apply_t_matrix, dtype=complex)

    def right_hand_side(self):
        """T_i a_i stacked over particles."""
        out = np.zeros(self.shape[0], dtype=complex)
        for i, p in enumerate(self.particle_list):
            out[int(self._offsets[i]):int(self._offsets[i + 1])] = p.t_matrix.dot(p.initial_field.coefficients)
        return out

    def device_blocks(self, blocksize, l_max, m_max):
        """Distinct T blocks embedded in the global lookup index space, and the type of each particle."""
        blocks = []
        keys = {}
        types = np.zeros(len(self.particle_list), dtype=np.int32)
        diagonal = True
        for i, p in enumerate(self.particle_list):
            t = p.t_matrix
            key = (p.l_max, p.m_max, t.tobytes())
            if key not in keys:
                tau, ll, mm = flds.index_table(p.l_max, p.m_max)
                gidx = np.array([flds.multi_to_single_index(a, b, c, l_max, m_max) for a, b, c in zip(tau, ll, mm)])
                full = np.zeros((blocksize, blocksize), complex)
                full[np.ix_(gidx, gidx)] = t
                keys[key] = len(blocks)
                blocks.append(full)
                diagonal &= bool(np.count_nonzero(t - np.diag(np.diag(t))) == 0)
            types[i] = keys[key]
        return np.array(blocks), types, diagonal


class MasterMatrix(SystemMatrix):
    """M = 1 - T W. With the GPU lookup, M v runs as one fused device operator."""

    def __init__(self, t_matrix, coupling_matrix):
        SystemMatrix.__init__(self, t_matrix.particle_list)
        self.t_matrix = t_matrix
        self.coupling_matrix = coupling_matrix
        if not isinstance(coupling_matrix, GPU_COUPLING_MATRICES):
            raise NotImplementedError('only the GPU lookup coupling matrices are provided by smuthi_gb300')
        blocks, types, diagonal = t_matrix.device_blocks(coupling_matrix.blocksize, coupling_matrix.l_max,
                                                         coupling_matrix.m_max)
        self.context = coupling_matrix.context
        self.context.set_tmatrix(blocks, types, diagonal)

        def apply_master_matrix(v):
            return self.context.master_matvec(np.asarray(v, dtype=complex).ravel(), coupling_matrix.precision)

        self.linear_operator = scipy.sparse.linalg.LinearOperator(shape=self.shape, matvec=apply_master_matrix,
                                                                  dtype=complex)


class LinearSystem:
    """Assemble and solve (1 - T W) b = T a with a GPU lookup (radial, or volume for particles at
    different heights).

    Extra keyword ``precision``: 'fp64' (plain drop-in, default) or 'mixed'
    (FP32 coupling operator inside FP64 iterative refinement; FP64 true
    residuals and FP64 Arnoldi). ``restart`` and ``maxiter`` are GMRES
    parameters with scipy's defaults (20, 10 x unknowns).
    """

    def __init__(self, particle_list, initial_field, layer_system, k_parallel='default', solver_type='LU',
                 solver_tolerance=1e-4, store_coupling_matrix=True, coupling_matrix_lookup_resolution=None,
                 interpolator_kind='cubic', cuda_blocksize=None, periodicity=None,
                 ewald_sum_separation_parameter='default', number_of_threads_periodic='default',
                 use_pvwf_coupling=False, pvwf_coupling_k_parallel=None, precision='fp64', restart=20, maxiter=None):
        self.particle_list = particle_list
        self.initial_field = initial_field
        self.layer_system = layer_system
        self.k_parallel = k_parallel
        self.solver_type = solver_type
        self.solver_tolerance = solver_tolerance
        self.store_coupling_matrix = store_coupling_matrix
        self.coupling_matrix_lookup_resolution = coupling_matrix_lookup_resolution
        self.interpolator_kind = interpolator_kind
        self.cuda_blocksize = cuda_blocksize if cuda_blocksize is not None else cu.default_blocksize
        self.periodicity = periodicity
        if precision not in PRECISIONS:
            raise ValueError("precision must be 'fp64' or 'mixed'")
        self.precision = precision
        self.restart = restart
        self.maxiter = maxiter
        self.solve_info = None
        sys.stdout.write('Number of unknowns: %i\n' % SystemMatrix(particle_list).shape[0])

    def prepare(self):
        self.compute_initial_field_coefficients()
        self.compute_t_matrix()
        self.compute_coupling_matrix()
        self.master_matrix = MasterMatrix(t_matrix=self.t_matrix, coupling_matrix=self.coupling_matrix)

    def compute_initial_field_coefficients(self):
        groups = {}
        for i, p in enumerate(self.particle_list):
            groups.setdefault((p.l_max, p.m_max, self.layer_system.layer_number(p.position[2])), []).append(i)
        for (lm, mm, layer), idx in groups.items():
            pos = np.array([self.particle_list[i].position for i in idx], dtype=float)
            coef = self.initial_field.swe_coefficients(pos, self.layer_system, lm, mm)
            k = self.initial_field.angular_frequency() * self.layer_system.refractive_indices[layer]
            for row, i in enumerate(idx):
                p = self.particle_list[i]
                swe = SphericalWaveExpansion(k=k, l_max=lm, m_max=mm, kind='regular', reference_point=p.position,
                                             lower_z=self.layer_system.lower_zlimit(layer),
                                             upper_z=self.layer_system.upper_zlimit(layer))
                swe.coefficients = coef[row]
                p.initial_field = swe

    def compute_t_matrix(self):
        for p in self.particle_list:
            n_med = self.layer_system.refractive_indices[self.layer_system.layer_number(p.position[2])]
            p.t_matrix = p.compute_t_matrix(self.initial_field.vacuum_wavelength, n_med)
            if p.euler_angles != [0, 0, 0]:
                raise NotImplementedError('rotated particles are outside the radial-lookup sphere path')
        self.t_matrix = TMatrix(particle_list=self.particle_list)

    def compute_coupling_matrix(self):
        if self.solver_type.lower() == 'lu' or self.store_coupling_matrix:
            raise NotImplementedError('smuthi_gb300 provides the lookup + GMRES path only: use solver_type="gmres", '
                                      'store_coupling_matrix=False and a coupling_matrix_lookup_resolution')
        if self.coupling_matrix_lookup_resolution is None:
            raise NotImplementedError('explicit coupling matrices are not provided; set a lookup resolution')
        if self.periodicity is not None:
            raise NotImplementedError('periodic particle arrangements are not provided by smuthi_gb300')
        layers_ = {self.layer_system.layer_number(p.position[2]) for p in self.particle_list}
        if len(layers_) != 1:
            raise NotImplementedError('particles in different layers need the explicit coupling path')
        z = {p.position[2] for p in self.particle_list}
        if not cu.use_gpu:
            raise RuntimeError('smuthi_gb300 has no CPU coupling path; GPU use is disabled')
        kind = self.interpolator_kind
        if kind not in ('linear', 'cubic', 'cubic_hermite'):
            warnings.warn(kind + ' interpolation not implemented. Use "linear" instead')
            kind = 'linear'
        if len(z) != 1:  # not all particles at one height: volume lookup (reference :206-215)
            sys.stdout.write('Coupling matrix computation by ' + kind + ' interpolation of 3D lookup on GPU.\n')
            self.coupling_matrix = CouplingMatrixVolumeLookupCUDA(
                vacuum_wavelength=self.initial_field.vacuum_wavelength, particle_list=self.particle_list,
                layer_system=self.layer_system, k_parallel=self.k_parallel,
                resolution=self.coupling_matrix_lookup_resolution, cuda_blocksize=self.cuda_blocksize,
                interpolator_kind=kind)
            return
        sys.stdout.write('Coupling matrix computation by ' + kind + ' interpolation of radial lookup on GPU.\n')
        self.coupling_matrix = CouplingMatrixRadialLookupCUDA(
            vacuum_wavelength=self.initial_field.vacuum_wavelength, particle_list=self.particle_list,
            layer_system=self.layer_system, k_parallel=self.k_parallel,
            resolution=self.coupling_matrix_lookup_resolution, cuda_blocksize=self.cuda_blocksize,
            interpolator_kind=kind)

    def solve(self):
        if len(self.particle_list) > 0:
            st = self.solver_type.lower()
            if st != 'gmres':
                raise NotImplementedError('solver_type %r is not provided (gmres only)' % self.solver_type)
            rhs = self.t_matrix.right_hand_side()
            start = time.time()
            ctx = self.coupling_matrix.context
            b, info = ctx.gmres(rhs, rhs, self.solver_tolerance, restart=self.restart, maxiter=self.maxiter or 0,
                                precision=PRECISIONS[self.precision], raise_on_failure=False)
            if info.converged < 1:
                # the reference ignores GMRES's info flag (linear_system.py:285); report it instead
                warnings.warn('GMRES did not reach the tolerance (rel. residual %.2e)' % info.max_rel_residual)
            self.solve_info = info.as_dict()
            sys.stdout.write('Solve (GMRES)             : Iter %d | Rel. residual: %.2e | elapsed: %ds\n'
                             % (info.iterations, info.max_rel_residual, int(time.time() - start)))
        for i, p in enumerate(self.particle_list):
            layer = self.layer_system.layer_number(p.position[2])
            k = flds.angular_frequency(self.initial_field.vacuum_wavelength) * self.layer_system.refractive_indices[
                layer]
            p.scattered_field = SphericalWaveExpansion(k=k, l_max=p.l_max, m_max=p.m_max, kind='outgoing',
                                                       reference_point=p.position,
                                                       lower_z=self.layer_system.lower_zlimit(layer),
                                                       upper_z=self.layer_system.upper_zlimit(layer))
            p.scattered_field.coefficients = b[self.master_matrix.index_block(i)]
            p.scattered_field.validity_conditions.append(p.is_outside)
            self.initial_field.validity_conditions.append(p.is_outside)
