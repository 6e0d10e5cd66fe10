"""GPU switch, mirroring ``smuthi.utility.cuda`` (smuthi/utility/cuda.py:5-68).

The reference falls back to its CPU classes when PyCUDA or the device probe
fails. This package has no CPU path: the radial-lookup coupling matrix always
runs on the GPU, and ``enable_gpu`` raises when no device can be opened.
"""
import sys

use_gpu = True
default_blocksize = 128


def enable_gpu(enable=True):
    """Set the ``use_gpu`` flag; with ``enable`` the device is probed once."""
    global use_gpu
    if not enable:
        use_gpu = False
        sys.stdout.write('Disabling GPU usage.\n')
        return
    from .._lib import Context
    ctx = Context(0)
    ctx.close()
    use_gpu = True
    sys.stdout.write('Enabling GPU usage.\n')
