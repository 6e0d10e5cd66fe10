"""Import the reference SMUTHI package in this container for fixture generation.

Three test-only shims make the reference importable with the installed
numpy/scipy and without numba:

* a pass-through ``numba`` package (``refshim/numba``);
* ``scipy.sparse.linalg.gmres`` accepting the removed ``tol=`` keyword
  (the reference calls ``gmres(M, rhs, rhs, tol=..., callback=...)`` at
  ``smuthi/linearsystem/linear_system.py:285``), forwarded as ``rtol=`` with
  ``callback_type='legacy'`` and ``atol=0`` (the pre-1.12 scipy defaults);
* ``np.trapz = np.trapezoid`` (used at ``smuthi/fields/transformations.py:126``
  and ``smuthi/postprocessing/far_field.py:108,127,138``).

The reference tree is read in place; nothing is copied from it.
"""
import os
import sys

import numpy as np
import scipy.sparse.linalg

REFERENCE_ROOT = os.environ.get("SMUTHI_REFERENCE_ROOT")  # the reference checkout that generates fixtures
_HERE = os.path.dirname(os.path.abspath(__file__))


def _install_shims():
    if not hasattr(np, "trapz"):
        np.trapz = np.trapezoid
    gm = scipy.sparse.linalg.gmres
    if not getattr(gm, "_smuthi_shim", False):
        def gmres(A, b, x0=None, *args, tol=None, callback=None, **kw):
            if tol is not None:
                kw.setdefault("rtol", tol)
            if callback is not None:
                kw.setdefault("callback_type", "legacy")
            kw.setdefault("atol", 0.0)
            return gm(A, b, x0, *args, callback=callback, **kw)
        gmres._smuthi_shim = True
        scipy.sparse.linalg.gmres = gmres


def import_reference():
    """Return the reference ``smuthi`` package (imported with the shims)."""
    if not REFERENCE_ROOT:
        raise RuntimeError("set SMUTHI_REFERENCE_ROOT to the reference source checkout (the directory holding "
                           "the smuthi package) to generate fixtures")
    if not os.path.isdir(os.path.join(REFERENCE_ROOT, "smuthi")):
        raise RuntimeError("reference source tree not found at " + REFERENCE_ROOT)
    shim = os.path.join(_HERE, "refshim")
    if shim not in sys.path:
        sys.path.insert(0, shim)
    if REFERENCE_ROOT not in sys.path:
        sys.path.insert(1, REFERENCE_ROOT)
    _install_shims()
    import smuthi  # noqa: F401
    import smuthi.simulation  # noqa: F401
    import smuthi.linearsystem.linear_system  # noqa: F401
    import smuthi.postprocessing.far_field  # noqa: F401
    return sys.modules["smuthi"]
