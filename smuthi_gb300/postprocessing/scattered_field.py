"""Plane-wave expansion of the scattered field (smuthi/postprocessing/scattered_field.py:80-150).

``scattered_field_pwe`` returns the upgoing and downgoing ``PlaneWaveExpansion`` of the particles'
scattered field in one layer, with the reference's reference point [0, 0, z_ref(layer)] and
validity bounds; its ``electric_field`` / ``magnetic_field`` evaluate the near field on the GPU.
The particle sum is the one of the cross sections (``far_field.scattered_pwe``): for particles in
one layer the per-particle conversions of the reference are summed as one matrix product before the
layer response is applied once.
"""
import numpy as np

from .. import fields as flds
from ..fields.expansions import PlaneWaveExpansion
from . import far_field


def scattered_field_pwe(vacuum_wavelength, particle_list, layer_system, layer_number, k_parallel='default',
                        azimuthal_angles='default', angular_resolution=None, include_direct=True,
                        include_layer_response=True, context=None):
    """(pwe_up, pwe_down) of the scattered field in ``layer_number`` (particles in one layer).

    ``context``: a library context for the particle sum on the GPU (used for real ``k_parallel``;
    the complex Sommerfeld contour is summed on the host).
    """
    if isinstance(k_parallel, str) and k_parallel == 'default':
        k_parallel = flds.default_Sommerfeld_k_parallel_array
    if angular_resolution is not None:
        azimuthal_angles, _ = flds.angular_arrays(angular_resolution)
    if isinstance(azimuthal_angles, str) and azimuthal_angles == 'default':
        azimuthal_angles = flds.default_azimuthal_angles
    if k_parallel is None or azimuthal_angles is None:
        raise ValueError('no default k_parallel / azimuthal angles: pass them or run a Simulation first')
    kpar = np.atleast_1d(np.asarray(k_parallel))
    alpha = np.atleast_1d(np.asarray(azimuthal_angles, dtype=float))
    layers_ = {layer_system.layer_number(p.position[2]) for p in particle_list}
    if len(layers_) != 1:
        raise NotImplementedError('the scattered-field expansion is provided for particles in one layer')
    omega = flds.angular_frequency(vacuum_wavelength)
    k = omega * layer_system.refractive_indices[layer_number]
    z_ref = layer_system.reference_z(layer_number)
    lo, hi = layer_system.lower_zlimit(layer_number), layer_system.upper_zlimit(layer_number)
    xy, z, l_max, m_max, coefs = far_field._particle_data(particle_list)
    real_kpar = not (np.iscomplexobj(kpar) and np.any(np.imag(kpar) != 0))
    g_up, g_dn = far_field.scattered_pwe(vacuum_wavelength, layer_system, xy, z, l_max, m_max, coefs, layer_number,
                                         kpar, alpha, context=context if real_kpar else None,
                                         include_direct=include_direct,
                                         include_layer_response=include_layer_response)
    # validity bounds as the reference's sums of per-particle expansions leave them (expansions.py:625-633)
    up_lo, dn_hi = lo, hi
    if include_direct and layers_.pop() == layer_number:
        zs = np.atleast_1d(z)
        up_lo, dn_hi = max(lo, float(np.max(zs))), min(hi, float(np.min(zs)))
    pwe_up = PlaneWaveExpansion(k=k, k_parallel=kpar, azimuthal_angles=alpha, kind='upgoing',
                                reference_point=[0, 0, z_ref], lower_z=up_lo, upper_z=hi)
    pwe_down = PlaneWaveExpansion(k=k, k_parallel=kpar, azimuthal_angles=alpha, kind='downgoing',
                                  reference_point=[0, 0, z_ref], lower_z=lo, upper_z=dn_hi)
    pwe_up.coefficients = g_up
    pwe_down.coefficients = g_dn
    return pwe_up, pwe_down
