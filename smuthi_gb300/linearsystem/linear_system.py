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
from .._lib import SG_DF64, SG_FP32, SG_FP64, SG_PRECOND, Context
from ..fields.expansions import SphericalWaveExpansion
from ..utility import cuda as cu
from .particlecoupling import prepare_lookup as look

PRECISIONS = {'fp64': SG_FP64, 'mixed': SG_FP32}
RESIDUALS = ('fp64', 'df64')


def shipped_preconditioner(layer_system, blocksize):
    """Name of the shipped learned-preconditioner weights for a layer system: those trained on the
    sphere film between two half-spaces for three or more layers, those trained on spheres above a
    substrate otherwise. Raises ValueError when no shipped weights fit the blocksize."""
    from .. import learned
    name = 'precond_c5' if layer_system.number_of_layers() >= 3 else 'precond_c2'
    learned.load_params(name, blocksize)  # checks the parameter count against the blocksize
    return name


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

    Extra keywords:

    * ``precision``: 'fp64' (plain drop-in, default) or 'mixed' (FP32 coupling
      operator inside FP64 iterative refinement, FP64 Arnoldi);
    * ``residual``: arithmetic of the mixed form's true residuals, 'fp64' (default) or
      'df64' (double-float on the FP32 pipe, FP64-grade);
    * ``preconditioner``: None (default), 'learned' (the shipped weights for the layer
      system, see ``shipped_preconditioner``) or the name of a weights file; mixed form
      with a radial lookup only (flexible GMRES with the learned right preconditioner);
    * ``initial_field`` may be a list of initial fields of one vacuum wavelength: their
      right-hand sides are solved as one batch and every particle gets one scattered
      field per initial field (``scattered_fields``; ``scattered_field`` is the first);
    * ``restart`` and ``maxiter`` are GMRES parameters with scipy's defaults (20, 10 x
      unknowns).

    The plain form starts GMRES at x0 = rhs like the reference; the mixed form at x0 = 0.
    """

    def __init__(self, particle_list, initial_field, layer_system, k_parallel='default', solver_type='LU',
                 solver_tolerance=1e-4, store_coupling_matrix=True, coupling_matrix_lookup_resolution=None,
                 interpolator_kind='cubic', cuda_blocksize=None, periodicity=None,
                 ewald_sum_separation_parameter='default', number_of_threads_periodic='default',
                 use_pvwf_coupling=False, pvwf_coupling_k_parallel=None, precision='fp64', restart=20, maxiter=None,
                 residual='fp64', preconditioner=None):
        self.particle_list = particle_list
        self.initial_fields = list(initial_field) if isinstance(initial_field, (list, tuple)) else [initial_field]
        if not self.initial_fields:
            raise ValueError('at least one initial field is needed')
        if len({f.vacuum_wavelength for f in self.initial_fields}) != 1:
            raise ValueError('initial fields solved as one batch must share the vacuum wavelength')
        self.initial_field = self.initial_fields[0]
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
        if residual not in RESIDUALS:
            raise ValueError("residual must be 'fp64' or 'df64'")
        if precision == 'fp64' and (residual != 'fp64' or preconditioner is not None):
            raise ValueError("residual='df64' and a preconditioner need precision='mixed'")
        self.precision = precision
        self.residual = residual
        self.preconditioner = preconditioner
        self.restart = restart
        self.maxiter = maxiter
        self.solve_info = None
        sys.stdout.write('Number of unknowns: %i\n' % SystemMatrix(particle_list).shape[0])

    def prepare(self):
        # the coupling matrix first: its GPU context also evaluates the initial fields at the particles
        self.compute_t_matrix()
        self.compute_coupling_matrix()
        self.compute_initial_field_coefficients(context=getattr(self.coupling_matrix, 'context', None))
        self.master_matrix = MasterMatrix(t_matrix=self.t_matrix, coupling_matrix=self.coupling_matrix)

    def compute_initial_field_coefficients(self, context=None):
        """Regular SWE of every initial field at every particle (``p.initial_fields``; ``p.initial_field``
        is the first). With a GPU context and plane-wave initial fields, all waves of a particle group are
        evaluated in one call of ``sg_plane_wave_swe``."""
        from ..initial_field import PlaneWave, swe_coefficients_batch
        groups = {}
        for i, p in enumerate(self.particle_list):
            groups.setdefault((p.l_max, p.m_max, self.layer_system.layer_number(p.position[2])), []).append(i)
            p.initial_fields = [None] * len(self.initial_fields)
        batch = {}
        if context is not None and all(isinstance(f, PlaneWave) for f in self.initial_fields):
            for key, idx in groups.items():
                pos = np.array([self.particle_list[i].position for i in idx], dtype=float)
                batch[key] = swe_coefficients_batch(self.initial_fields, pos, self.layer_system, key[0], key[1],
                                                    context)
        for q, field in enumerate(self.initial_fields):
            for (lm, mm, layer), idx in groups.items():
                pos = np.array([self.particle_list[i].position for i in idx], dtype=float)
                coef = batch[(lm, mm, layer)][q] if batch else field.swe_coefficients(pos, self.layer_system, lm, mm)
                k = field.angular_frequency() * self.layer_system.refractive_indices[layer]
                for row, i in enumerate(idx):
                    p = self.particle_list[i]
                    swe = SphericalWaveExpansion(k=k, l_max=lm, m_max=mm, kind='regular', reference_point=p.position,
                                                 lower_z=self.layer_system.lower_zlimit(layer),
                                                 upper_z=self.layer_system.upper_zlimit(layer))
                    swe.coefficients = coef[row]
                    p.initial_fields[q] = swe
        for p in self.particle_list:
            p.initial_field = p.initial_fields[0]

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
            cols = []
            for q in range(len(self.initial_fields)):
                for p in self.particle_list:
                    p.initial_field = p.initial_fields[q]
                cols.append(self.t_matrix.right_hand_side())
            for p in self.particle_list:
                p.initial_field = p.initial_fields[0]
            nrhs = len(cols)
            rhs = cols[0] if nrhs == 1 else np.ascontiguousarray(np.stack(cols, axis=1))
            start = time.time()
            ctx = self.coupling_matrix.context
            flags = PRECISIONS[self.precision]
            if self.precision == 'mixed':
                if self.residual == 'df64':
                    flags |= SG_DF64
                if self.preconditioner is not None:
                    self._attach_preconditioner(ctx)
                    flags |= SG_PRECOND
            x0 = rhs if self.precision == 'fp64' else np.zeros_like(rhs)
            b, info = ctx.gmres(rhs, x0, self.solver_tolerance, restart=self.restart, maxiter=self.maxiter or 0,
                                precision=flags, raise_on_failure=False)
            if info.converged < nrhs:
                # the reference ignores GMRES's info flag (linear_system.py:285); report it instead
                warnings.warn('GMRES did not reach the tolerance (rel. residual %.2e)' % info.max_rel_residual)
            self.solve_info = info.as_dict()
            sys.stdout.write('Solve (GMRES)             : Iter %d | Rel. residual: %.2e | elapsed: %ds\n'
                             % (info.iterations, info.max_rel_residual, int(time.time() - start)))
            B = b.reshape(-1, 1) if b.ndim == 1 else b
        else:
            B = np.zeros((0, len(self.initial_fields)), complex)
        for i, p in enumerate(self.particle_list):
            layer = self.layer_system.layer_number(p.position[2])
            k = flds.angular_frequency(self.initial_field.vacuum_wavelength) * self.layer_system.refractive_indices[
                layer]
            p.scattered_fields = []
            for q in range(len(self.initial_fields)):
                swe = SphericalWaveExpansion(k=k, l_max=p.l_max, m_max=p.m_max, kind='outgoing',
                                             reference_point=p.position, lower_z=self.layer_system.lower_zlimit(layer),
                                             upper_z=self.layer_system.upper_zlimit(layer))
                swe.coefficients = B[self.master_matrix.index_block(i), q]
                swe.validity_conditions.append(p.is_outside)
                p.scattered_fields.append(swe)
            p.scattered_field = p.scattered_fields[0]
            for field in self.initial_fields:
                field.validity_conditions.append(p.is_outside)

    def _attach_preconditioner(self, ctx):
        """Select the learned preconditioner on the context (radial lookup, uniform particles)."""
        from .. import learned
        cm = self.coupling_matrix
        if not isinstance(cm, CouplingMatrixRadialLookupCUDA):
            raise NotImplementedError('the learned preconditioner serves the radial lookup only')
        bs = cm.blocksize
        name = shipped_preconditioner(self.layer_system, bs) if self.preconditioner == 'learned' \
            else self.preconditioner
        xy = np.array([p.position[:2] for p in self.particle_list], dtype=float)
        learned.attach(ctx, xy, bs, learned.load_params(name, bs), k=learned.load_meta(name)['k'])
        self.preconditioner_name = name
