"""CPU oracle for the SMUTHI radial-lookup coupling solve path.

TEST INFRASTRUCTURE ONLY. This package is a plain numpy/scipy restatement of
the reference algorithm (somso2e/smuthi v2.1.2) for the particle-coupling
solve path: SVWF indexing, the Sommerfeld contour, layer response, Mie
T-matrices, plane-wave right-hand sides, the radial coupling lookup table,
the CPU lookup matvec (``CouplingMatrixRadialLookupCPU``), the master
operator, scipy GMRES and the extinction / total scattering cross sections.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg (and its ``--impl reference`` arm) may import it, and only as the
values a test compares against or as the timed CPU baseline. The product package ``smuthi_gb300``
never imports it and has no CPU fallback.

Parity pin: the oracle is checked against (a) golden vectors generated by
running the reference itself in the build container (``tests/golden/``,
generating script committed beside them) and (b) the known-answer values
hard-coded in the reference's own unit tests.

Third-party arithmetic the reference relies on (not in the reference tree):
scipy (``interp1d``, ``gmres``, ``special.jv``, ``spherical_jn/yn``), sympy
(``wigner_3j``; restated here as the exact Racah formula) and numpy.
"""
