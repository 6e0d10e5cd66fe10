"""smuthi_gb300: GB300-native (sm_103a) particle-coupling solve path of SMUTHI.

A drop-in for SMUTHI's ``CouplingMatrixRadialLookupCUDA`` (particles at one
height), ``CouplingMatrixVolumeLookupCUDA`` (particles at different heights in
one layer) and the GMRES loop that drives them, with the cross sections and the
near field of plane-wave expansions on the GPU. The module tree mirrors
``smuthi`` (``simulation``, ``layers``, ``particles``, ``initial_field``,
``fields``, ``linearsystem.linear_system``, ``postprocessing.far_field``,
``postprocessing.scattered_field``, ``utility.cuda``) so that
``import smuthi_gb300 as smuthi`` keeps user scripts running. Compute runs only
through the in-tree CUDA library (``libsmuthi_gb300.so``, C ABI in
``include/smuthi_gb300.h``).
"""
__version__ = "0.1.0"
