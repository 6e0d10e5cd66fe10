"""Simulation driver mirroring smuthi/simulation.py (:92-153 constructor, :363-414 run).

Same keyword arguments as the reference. Extra keywords select the solve form:

* ``precision``: the plain FP64 drop-in ('fp64', default) or the mixed-precision form ('mixed':
  FP32 coupling operator inside FP64 iterative refinement);
* ``residual``: the mixed form's true residuals in FP64 ('fp64', default) or in FP64-grade
  double-float arithmetic on the FP32 pipe ('df64');
* ``preconditioner``: None, 'learned' (the shipped learned right preconditioner for the layer
  system) or a weights-file name;
* ``initial_field`` may be a list of plane waves of one wavelength, solved as one batch: after
  ``run`` every particle holds ``scattered_fields`` (one per wave) and ``select_wave(q)`` makes wave
  q the simulation's ``initial_field`` and each particle's ``scattered_field`` (what the
  post-processing functions read).

The chosen form of this package is ``precision='mixed', residual='df64',
preconditioner='learned'`` with several plane waves. ``run`` returns (preparation, solution,
post-processing) seconds.
"""
import sys
import time
import warnings

import numpy as np

from . import fields as flds
from .linearsystem import linear_system as lsys


class Simulation:
    def __init__(self, layer_system=None, particle_list=None, initial_field=None, k_parallel='default',
                 angular_resolution=np.pi / 360, neff_waypoints=None, neff_imag=1e-2, neff_max=None,
                 neff_max_offset=1, neff_resolution=1e-2, neff_minimal_branchpoint_distance=None,
                 overwrite_default_contours=True, solver_type='LU', solver_tolerance=1e-4,
                 store_coupling_matrix=True, coupling_matrix_lookup_resolution=None,
                 coupling_matrix_interpolator_kind='linear', length_unit='length unit', input_file=None,
                 output_dir='smuthi_output', save_after_run=False, log_to_file=False, log_to_terminal=True,
                 check_circumscribing_spheres=True, do_sanity_check=True, periodicity=None,
                 ewald_sum_separation_parameter='default', number_of_threads_periodic='default',
                 use_pvwf_coupling=False, pvwf_coupling_neff_max=None, pvwf_coupling_neff_resolution=1e-2,
                 precision='fp64', restart=20, maxiter=None, residual='fp64', preconditioner=None):
        self.layer_system = layer_system
        self.particle_list = particle_list
        self.initial_fields = list(initial_field) if isinstance(initial_field, (list, tuple)) else [initial_field]
        self.initial_field = self.initial_fields[0]
        self.k_parallel = k_parallel
        self.angular_resolution = angular_resolution
        self.neff_waypoints = neff_waypoints
        self.neff_imag = neff_imag
        self.neff_max = neff_max
        self.neff_max_offset = neff_max_offset
        self.neff_resolution = neff_resolution
        self.neff_minimal_branchpoint_distance = neff_minimal_branchpoint_distance
        self.overwrite_default_contours = overwrite_default_contours
        self.solver_type = solver_type
        self.solver_tolerance = solver_tolerance
        self.store_coupling_matrix = store_coupling_matrix
        self.coupling_matrix_lookup_resolution = coupling_matrix_lookup_resolution
        self.coupling_matrix_interpolator_kind = coupling_matrix_interpolator_kind
        self.length_unit = length_unit
        self.log_to_terminal = log_to_terminal
        self.check_circumscribing_spheres = check_circumscribing_spheres
        self.do_sanity_check = do_sanity_check
        self.periodicity = periodicity
        if use_pvwf_coupling:
            raise NotImplementedError('plane-wave coupling is not part of the radial-lookup path')
        self.precision = precision
        self.residual = residual
        self.preconditioner = preconditioner
        self.restart = restart
        self.maxiter = maxiter
        self.post_processing = None
        self.linear_system = None

    def _write(self, msg):
        if self.log_to_terminal:
            sys.stdout.write(msg)

    def largest_lateral_distance(self):
        xy = np.array([p.position[:2] for p in self.particle_list], dtype=float)
        lo, hi = xy.min(0), xy.max(0)
        # exact max pairwise distance needs O(N^2); the hull diagonal bounds it from above, used only as a hint
        best = 0.0
        for s in range(0, len(xy), 2048):
            blk = xy[s:s + 2048]
            d2 = ((blk[:, None, :] - xy[None, :, :]) ** 2).sum(-1)
            best = max(best, float(d2.max()))
        del lo, hi
        return np.sqrt(best)

    def sanity_check(self):
        """smuthi/simulation.py:223-251: warn if the contour resolution is too coarse for the geometry."""
        maxrho = self.largest_lateral_distance()
        k = flds.angular_frequency(self.initial_field.vacuum_wavelength)
        thresh = 2 / (maxrho * k)
        if self.neff_resolution is not None and isinstance(self.k_parallel, str) and self.neff_resolution > thresh:
            self._write("Warning: Sanity check for neff_resolution failed! neff_resolution = %.3e, "
                        "recommended < %.3e\n" % (self.neff_resolution, thresh))
        if (self.neff_imag is not None and isinstance(self.k_parallel, str) and self.neff_waypoints is None
                and self.neff_imag > thresh):
            self._write("Warning: Sanity check for neff_imag failed! neff_imag = %.3e, recommended < %.3e\n"
                        % (self.neff_imag, thresh))

    def circumscribing_spheres_disjoint(self):
        """True if no two circumscribing spheres overlap (cell-list check, O(N))."""
        pos = np.array([p.position for p in self.particle_list], dtype=float)
        rad = np.array([p.circumscribing_sphere_radius() for p in self.particle_list], dtype=float)
        cell = 2 * rad.max()
        keys = np.floor(pos / cell).astype(np.int64)
        grid = {}
        for i, k in enumerate(map(tuple, keys)):
            grid.setdefault(k, []).append(i)
        for i, k in enumerate(map(tuple, keys)):
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dz in (-1, 0, 1):
                        for j in grid.get((k[0] + dx, k[1] + dy, k[2] + dz), ()):
                            if j > i and np.sum((pos[i] - pos[j]) ** 2) < (rad[i] + rad[j]) ** 2:
                                self._write('The circumscribing sphere of particle %i overlaps with that of '
                                            'particle %i.\n' % (i, j))
                                return False
        return True

    def set_default_Sommerfeld_contour(self):
        flds.default_Sommerfeld_k_parallel_array = flds.reasonable_Sommerfeld_kpar_contour(
            vacuum_wavelength=self.initial_field.vacuum_wavelength, neff_waypoints=self.neff_waypoints,
            layer_refractive_indices=self.layer_system.refractive_indices, neff_imag=self.neff_imag,
            neff_max=self.neff_max, neff_max_offset=self.neff_max_offset, neff_resolution=self.neff_resolution,
            neff_minimal_branchpoint_distance=self.neff_minimal_branchpoint_distance)

    def set_default_angles(self):
        flds.default_azimuthal_angles, flds.default_polar_angles = flds.angular_arrays(self.angular_resolution)

    def select_wave(self, q):
        """Make initial field q (of a batch) the simulation's ``initial_field`` and every particle's
        ``initial_field`` and ``scattered_field`` that of wave q (the post-processing reads these)."""
        self.initial_field = self.initial_fields[q]
        for p in self.particle_list:
            if getattr(p, 'initial_fields', None):
                p.initial_field = p.initial_fields[q]
            if getattr(p, 'scattered_fields', None):
                p.scattered_field = p.scattered_fields[q]

    def initialize_linear_system(self):
        self.linear_system = lsys.LinearSystem(
            particle_list=self.particle_list,
            initial_field=self.initial_fields if len(self.initial_fields) > 1 else self.initial_field,
            layer_system=self.layer_system,
            k_parallel=self.k_parallel, solver_type=self.solver_type, solver_tolerance=self.solver_tolerance,
            store_coupling_matrix=self.store_coupling_matrix,
            coupling_matrix_lookup_resolution=self.coupling_matrix_lookup_resolution,
            interpolator_kind=self.coupling_matrix_interpolator_kind, periodicity=self.periodicity,
            precision=self.precision, restart=self.restart, maxiter=self.maxiter, residual=self.residual,
            preconditioner=self.preconditioner)

    def run(self):
        """Prepare and solve; returns (preparation_time, solution_time, postprocessing_time)."""
        stdout = sys.stdout
        if not self.log_to_terminal:
            sys.stdout = _Null()
        try:
            if self.check_circumscribing_spheres and len(self.particle_list) > 1 \
                    and not self.circumscribing_spheres_disjoint():
                warnings.warn("Particles with circumscribing spheres detected.")
            if self.do_sanity_check and len(self.particle_list) > 1:
                self.sanity_check()
            if flds.default_azimuthal_angles is None or flds.default_polar_angles is None:
                self.set_default_angles()
            if flds.default_Sommerfeld_k_parallel_array is None or self.overwrite_default_contours:
                self.set_default_Sommerfeld_contour()
            t0 = time.time()
            self.initialize_linear_system()
            self.linear_system.prepare()
            t1 = time.time()
            self.linear_system.solve()
            t2 = time.time()
            if self.post_processing:
                self.post_processing.run(self)
            t3 = time.time()
        finally:
            sys.stdout = stdout
        return t1 - t0, t2 - t1, t3 - t2


class _Null:
    def write(self, *a):
        pass

    def flush(self):
        pass
