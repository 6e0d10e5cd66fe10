"""SVWF indexing, wave-vector helpers and default contours.

Mirrors smuthi/fields/__init__.py: the multi index n(tau, l, m) (:29-80),
``blocksize`` (:83-94), ``k_z`` (:101-129), the Sommerfeld contour
construction (:153-370) and the default angular arrays (:132-150).
"""
import numpy as np


def angular_frequency(vacuum_wavelength):
    """omega = 2 pi / lambda in units of c = 1 (also the vacuum wavenumber)."""
    return 2 * np.pi / vacuum_wavelength


def multi_to_single_index(tau, l, m, l_max, m_max):
    """Position of (tau, l, m) in a particle's coefficient block."""
    per_tau = m_max * (m_max + 2) + (l_max - m_max) * (2 * m_max + 1)
    if l - 1 <= m_max:
        before = (l - 1) * (l + 1)
    else:
        before = m_max * (m_max + 2) + (l - 1 - m_max) * (2 * m_max + 1)
    return tau * per_tau + before + m + min(l, m_max)


def blocksize(l_max, m_max):
    """Number of (tau, l, m) coefficients of one particle."""
    return 2 * (m_max * (m_max + 2) + (l_max - m_max) * (2 * m_max + 1))


def index_table(l_max, m_max):
    """Arrays (tau, l, m) indexed by the multi index n."""
    bs = blocksize(l_max, m_max)
    tau = np.zeros(bs, int)
    ll = np.zeros(bs, int)
    mm = np.zeros(bs, int)
    for t in range(2):
        for l in range(1, l_max + 1):
            for m in range(-min(l, m_max), min(l, m_max) + 1):
                n = multi_to_single_index(t, l, m, l_max, m_max)
                tau[n], ll[n], mm[n] = t, l, m
    return tau, ll, mm


def k_z(k_parallel=None, n_effective=None, k=None, omega=None, vacuum_wavelength=None, refractive_index=None):
    """sqrt(k^2 - kappa^2) on the branch with non-negative imaginary part."""
    if k_parallel is None:
        if omega is None:
            omega = angular_frequency(vacuum_wavelength)
        k_parallel = n_effective * omega
    if k is None:
        if omega is None:
            omega = angular_frequency(vacuum_wavelength)
        k = refractive_index * omega
    kz = np.sqrt(k ** 2 - np.asarray(k_parallel) ** 2 + 0j)
    return np.where(kz.imag < 0, -kz, kz)


def angular_arrays(angular_resolution=np.pi / 360):
    """(azimuthal, polar) angle arrays with the given step."""
    az = np.arange(0, 2 * np.pi + 0.5 * angular_resolution, angular_resolution, dtype=float)
    po = np.arange(0, np.pi + 0.5 * angular_resolution, angular_resolution, dtype=float)
    return az, po


default_azimuthal_angles = None
default_polar_angles = None
default_Sommerfeld_k_parallel_array = None
default_initial_field_k_parallel_array = None


def reasonable_neff_waypoints(layer_refractive_indices=None, neff_imag=1e-2, neff_max=None, neff_max_offset=1):
    """Contour corners that detour below the real axis around mode/branch-point positions."""
    if layer_refractive_indices is None:
        layer_refractive_indices = [1, 2]
    real_n = np.array(layer_refractive_indices).real
    lo = max(0, min(real_n) - 0.1)
    hi = max(real_n) + 0.2
    if neff_max is None:
        neff_max = hi + neff_max_offset
    if neff_imag == 0:
        return [0, neff_max]
    pts = [0, lo, lo - 1j * neff_imag, hi - 1j * neff_imag, hi]
    if neff_max > hi:
        pts.append(neff_max)
    return pts


def create_neff_array(neff_waypoints, neff_resolution):
    """Sample the polygonal contour through the waypoints at the given spacing."""
    pieces = []
    for a, b in zip(neff_waypoints[:-1], neff_waypoints[1:]):
        d = abs(b - a)
        if d > 0:
            cnt = int(np.ceil(d / neff_resolution)) + 1
            pieces.append(a + np.linspace(0, 1, num=cnt, endpoint=True, dtype=complex) * (b - a))
    return np.concatenate(pieces)


def branchpoint_correction(layer_refractive_indices, n_effective_array, neff_minimal_branchpoint_distance):
    """Replace samples that sit on a branch point by midpoints towards their neighbours."""
    arr = n_effective_array
    for n in layer_refractive_indices:
        while True:
            near = np.flatnonzero(abs(arr - n) < neff_minimal_branchpoint_distance)
            if near.size == 0:
                break
            i = near[0]
            if i != len(arr) - 1:
                arr = np.insert(arr, i + 1, (arr[i] + arr[i + 1]) / 2.0)
                if abs(arr[i + 1] - n) < neff_minimal_branchpoint_distance:
                    arr = np.delete(arr, i + 1)
            if i != 0:
                arr[i] = (arr[i - 1] + arr[i]) / 2.0
                if abs(arr[i] - n) < neff_minimal_branchpoint_distance:
                    arr = np.delete(arr, i)
    return arr


def reasonable_Sommerfeld_neff_contour(neff_waypoints=None, layer_refractive_indices=None, neff_imag=1e-2,
                                       neff_max=None, neff_max_offset=1, neff_resolution=1e-2,
                                       neff_minimal_branchpoint_distance=None):
    if neff_waypoints is None:
        neff_waypoints = reasonable_neff_waypoints(layer_refractive_indices, neff_imag, neff_max, neff_max_offset)
    if neff_minimal_branchpoint_distance is None:
        neff_minimal_branchpoint_distance = neff_resolution / 5
    arr = create_neff_array(neff_waypoints, neff_resolution)
    if layer_refractive_indices is not None:
        arr = branchpoint_correction(layer_refractive_indices, arr, neff_minimal_branchpoint_distance)
    return arr


def reasonable_Sommerfeld_kpar_contour(vacuum_wavelength, neff_waypoints=None, layer_refractive_indices=None,
                                       neff_imag=1e-2, neff_max=None, neff_max_offset=1, neff_resolution=1e-2,
                                       neff_minimal_branchpoint_distance=None):
    """In-plane wavenumber contour for Sommerfeld integrals."""
    return reasonable_Sommerfeld_neff_contour(neff_waypoints, layer_refractive_indices, neff_imag, neff_max,
                                              neff_max_offset, neff_resolution,
                                              neff_minimal_branchpoint_distance) * angular_frequency(vacuum_wavelength)
