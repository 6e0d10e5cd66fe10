"""ctypes binding of the in-tree CUDA library ``libsmuthi_gb300.so``.

The library is the only compute path of this package: there is no CPU
fallback. ``lib()`` raises ``LibraryMissing`` when the shared object has not
been built (``python -m smuthi_gb300.build``) and every wrapped call raises
``SmuthiGB300Error`` with the library's message when it returns a non-zero
status.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsmuthi_gb300.so")

SG_OK, SG_ERR_ARG, SG_ERR_CUDA, SG_ERR_NOT_CONVERGED, SG_ERR_NAN, SG_ERR_NO_DEVICE = range(6)
SG_LINEAR, SG_CUBIC, SG_CUBIC_HERMITE = 0, 1, 2
SG_FP64, SG_FP32 = 0, 1
SG_BLOCK_GMRES = 2  # OR-ed with SG_FP32: block GMRES correction solves
SG_PRECOND = 4  # OR-ed with SG_FP32: flexible GMRES corrections with the learned preconditioner
SG_DF64 = 8  # double-float operator; OR-ed with SG_FP32: refinement residuals in double-float
SG_TF32X3 = 16  # FP32-grade operator on the tensor cores (3xTF32), batched RHS
KINDS = {"linear": SG_LINEAR, "cubic": SG_CUBIC, "cubic_hermite": SG_CUBIC_HERMITE}

#: every entry point declared in include/smuthi_gb300.h
EXPORTS = ("sg_last_error", "sg_version", "sg_create", "sg_destroy", "sg_set_particles", "sg_set_lookup",
           "sg_set_tmatrix", "sg_coupling_matvec", "sg_master_matvec", "sg_coupling_matvec_dev",
           "sg_master_matvec_dev", "sg_gmres_solve", "sg_gmres_solve_dev", "sg_true_residual", "sg_profile",
           "sg_kernel_timing", "sg_launch_count", "sg_measure_fma_peak", "sg_fp32_autotune", "sg_fp32_set_kernel",
           "sg_tc_set_window", "sg_coupling_matvec_linear_noalloc", "sg_precond_param_count", "sg_precond_add_graph",
           "sg_precond_select", "sg_precond_clear", "sg_precond_set_params", "sg_precond_get_params",
           "sg_precond_apply_dev", "sg_precond_train_step", "sg_precond_export_blocks", "sg_bessel_jac_table",
           "sg_lookup_contract", "sg_plane_wave_swe",
           "sg_farfield_sum", "sg_set_volume_lookup", "sg_farfield_sum_heights", "sg_pwe_field")


class LibraryMissing(RuntimeError):
    pass


class SmuthiGB300Error(RuntimeError):
    def __init__(self, code, message):
        super().__init__("smuthi_gb300 error %d: %s" % (code, message))
        self.code = code


class NotConverged(SmuthiGB300Error):
    pass


class SolveInfo(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("restarts", ctypes.c_int32), ("fp64_matvecs", ctypes.c_int32),
                ("fp32_matvecs", ctypes.c_int32), ("converged", ctypes.c_int32),
                ("precond_fallbacks", ctypes.c_int32),
                ("max_rel_residual", ctypes.c_double), ("seconds", ctypes.c_double),
                ("device_seconds", ctypes.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_LIB = None
_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double


def _declare(L):
    L.sg_last_error.restype = ctypes.c_char_p
    L.sg_version.restype = ctypes.c_char_p
    sigs = {
        "sg_create": [_I, ctypes.POINTER(_P)],
        "sg_destroy": [_P],
        "sg_set_particles": [_P, _I, _P, _I, _P, _P, _I, _P],
        "sg_set_lookup": [_P, _I, _I, _D, _D, _P],
        "sg_set_volume_lookup": [_P, _I, _P, _I, _D, _I, _D, _D, _D, _P, _P],
        "sg_set_tmatrix": [_P, _I, _P, _P, _I],
        "sg_coupling_matvec": [_P, _P, _P, _I, _I],
        "sg_master_matvec": [_P, _P, _P, _I, _I],
        "sg_coupling_matvec_dev": [_P, _P, _P, _I, _I, _P],
        "sg_master_matvec_dev": [_P, _P, _P, _I, _I, _P],
        "sg_gmres_solve": [_P, _P, _P, _I, _D, _I, _I, _I, ctypes.POINTER(SolveInfo)],
        "sg_gmres_solve_dev": [_P, _P, _P, _I, _D, _I, _I, _I, ctypes.POINTER(SolveInfo), _P],
        "sg_true_residual": [_P, _P, _P, _I, _P],
        "sg_profile": [_P, _I],
        "sg_kernel_timing": [_P, _I, ctypes.POINTER(_D), ctypes.POINTER(ctypes.c_int64), _I],
        "sg_launch_count": [_P, ctypes.POINTER(ctypes.c_int64)],
        "sg_measure_fma_peak": [_P, _I, ctypes.POINTER(_D)],
        "sg_fp32_autotune": [_P, _I, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_D), ctypes.POINTER(_D),
                             ctypes.POINTER(_D), ctypes.POINTER(_D), ctypes.POINTER(_D)],
        "sg_fp32_set_kernel": [_P, _I, _I, _I],
        "sg_tc_set_window": [_P, _I],
        "sg_plane_wave_swe": [_P, _I, _P, _I, _I, _P, _I, _P, _P, _P],
        "sg_coupling_matvec_linear_noalloc": [_I, _I, _P, _I, _P, _I, _D, _D, _P, _P, _P, _I, _P],
        "sg_bessel_jac_table": [_P, _P, _P, _I, _P, _I, _I, _P, _P],
        "sg_lookup_contract": [_P, _P, _I, _I, _P, _I, _P, _D, _D, _P, ctypes.c_longlong, _P],
        "sg_farfield_sum": [_P, _I, _P, _I, _I, _P, _I, _P, _I, _P, _P, _I, _P, _P, _P],
        "sg_farfield_sum_heights": [_P, _I, _P, _I, _I, _P, _I, _P, _I, _P, _P, _I, _P, _P, _P, _P],
        "sg_pwe_field": [_P, _I, _I, _P, _P, _P, _I, _P, _P, _I, _P, _P, _D, _D, _D, _P, _P],
        "sg_precond_param_count": [_I],
        "sg_precond_add_graph": [_P, _I, _P, ctypes.POINTER(_I)],
        "sg_precond_select": [_P, _I],
        "sg_precond_clear": [_P],
        "sg_precond_set_params": [_P, _I, _P, _I],
        "sg_precond_get_params": [_P, _P, _I],
        "sg_precond_apply_dev": [_P, _P, _P, _I, _P],
        "sg_precond_train_step": [_P, _I, _P, _P, _I, ctypes.c_float, _I, ctypes.POINTER(_D), _P],
        "sg_precond_export_blocks": [_P, _I, _P],
    }
    for name, args in sigs.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = _I


def lib():
    """Load (once) and return the ctypes library handle."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise LibraryMissing("CUDA library not built: %s is missing (run python -m smuthi_gb300.build)"
                                 % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        _declare(L)
        _LIB = L
    return _LIB


def check(rc):
    if rc != SG_OK:
        msg = lib().sg_last_error().decode(errors="replace")
        if rc == SG_ERR_NOT_CONVERGED:
            raise NotConverged(rc, msg)
        raise SmuthiGB300Error(rc, msg)


def ptr(a):
    """Pointer to the data of a C-contiguous numpy array."""
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return ctypes.c_void_p(a.ctypes.data)


class Context:
    """Owns one ``sg_context`` on a CUDA device."""

    def __init__(self, device=0):
        L = lib()
        h = ctypes.c_void_p()
        check(L.sg_create(device, ctypes.byref(h)))
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            lib().sg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- uploads
    def set_particles(self, xy, unknown_particle, unknown_n, blocksize, m_of_n):
        xy = np.ascontiguousarray(xy, dtype=np.float64)
        up = np.ascontiguousarray(unknown_particle, dtype=np.int32)
        un = np.ascontiguousarray(unknown_n, dtype=np.int32)
        mo = np.ascontiguousarray(m_of_n, dtype=np.int32)
        check(lib().sg_set_particles(self.h, xy.shape[0], ptr(xy), len(up), ptr(up), ptr(un), int(blocksize),
                                     ptr(mo)))

    def set_lookup(self, kind, table, rho_min, resolution):
        tab = np.ascontiguousarray(table, dtype=np.complex128)
        check(lib().sg_set_lookup(self.h, KINDS[kind] if isinstance(kind, str) else int(kind), tab.shape[0],
                                  float(rho_min), float(resolution), ptr(tab)))

    def set_volume_lookup(self, kind, z, table_plus, table_minus, rho_min, sz_min, dz_min, resolution):
        """Volume lookup [rho, z, n1, n2] tables (z1 + z2 and z1 - z2) and the particle heights."""
        zz = np.ascontiguousarray(z, dtype=np.float64)
        tp = np.ascontiguousarray(table_plus, dtype=np.complex128)
        tm = np.ascontiguousarray(table_minus, dtype=np.complex128)
        if tp.shape != tm.shape or tp.ndim != 4:
            raise ValueError("volume tables must both be [len_rho, len_z, blocksize, blocksize]")
        check(lib().sg_set_volume_lookup(self.h, KINDS[kind] if isinstance(kind, str) else int(kind), ptr(zz),
                                         tp.shape[0], float(rho_min), tp.shape[1], float(sz_min), float(dz_min),
                                         float(resolution), ptr(tp), ptr(tm)))

    def set_tmatrix(self, blocks, particle_type, diagonal):
        t = np.ascontiguousarray(blocks, dtype=np.complex128)
        pt = np.ascontiguousarray(particle_type, dtype=np.int32)
        check(lib().sg_set_tmatrix(self.h, t.shape[0], ptr(t), ptr(pt), 1 if diagonal else 0))

    # -- operators (host buffers)
    def _matvec(self, fn, x, precision):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        nrhs = 1 if x.ndim == 1 else x.shape[1]
        y = np.empty_like(x)
        check(fn(self.h, ptr(x), ptr(y), nrhs, precision))
        return y

    def coupling_matvec(self, x, precision=SG_FP64):
        return self._matvec(lib().sg_coupling_matvec, x, precision)

    def master_matvec(self, x, precision=SG_FP64):
        return self._matvec(lib().sg_master_matvec, x, precision)

    def gmres(self, b, x0, rtol, restart=20, maxiter=0, precision=SG_FP64, raise_on_failure=True):
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.array(x0, dtype=np.complex128, order="C", copy=True)
        nrhs = 1 if b.ndim == 1 else b.shape[1]
        info = SolveInfo()
        rc = lib().sg_gmres_solve(self.h, ptr(b), ptr(x), nrhs, float(rtol), int(restart), int(maxiter),
                                  int(precision), ctypes.byref(info))
        if rc != SG_OK and (raise_on_failure or rc != SG_ERR_NOT_CONVERGED):
            check(rc)
        return x, info

    def gmres_dev(self, b_ptr, x_ptr, nrhs, rtol, restart=20, maxiter=0, precision=SG_FP64, stream=None):
        info = SolveInfo()
        rc = lib().sg_gmres_solve_dev(self.h, ctypes.c_void_p(b_ptr), ctypes.c_void_p(x_ptr), int(nrhs),
                                      float(rtol), int(restart), int(maxiter), int(precision), ctypes.byref(info),
                                      ctypes.c_void_p(stream or 0))
        if rc not in (SG_OK, SG_ERR_NOT_CONVERGED):
            check(rc)
        return info

    def master_matvec_dev(self, x_ptr, y_ptr, nrhs, precision=SG_FP64, stream=None):
        check(lib().sg_master_matvec_dev(self.h, ctypes.c_void_p(x_ptr), ctypes.c_void_p(y_ptr), int(nrhs),
                                         int(precision), ctypes.c_void_p(stream or 0)))

    def coupling_matvec_dev(self, x_ptr, y_ptr, nrhs, precision=SG_FP64, stream=None):
        check(lib().sg_coupling_matvec_dev(self.h, ctypes.c_void_p(x_ptr), ctypes.c_void_p(y_ptr), int(nrhs),
                                           int(precision), ctypes.c_void_p(stream or 0)))

    def true_residual(self, b, x):
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.ascontiguousarray(x, dtype=np.complex128)
        nrhs = 1 if b.ndim == 1 else b.shape[1]
        out = np.zeros(nrhs)
        check(lib().sg_true_residual(self.h, ptr(b), ptr(x), nrhs, ptr(out)))
        return out

    # -- instrumentation
    def profile(self, enable=True):
        check(lib().sg_profile(self.h, 1 if enable else 0))

    def kernel_timing(self, precision=-1, reset=True):
        """(summed ms, launches) of profiled coupling kernels of a precision (-1: both)."""
        ms = ctypes.c_double()
        n = ctypes.c_int64()
        check(lib().sg_kernel_timing(self.h, int(precision), ctypes.byref(ms), ctypes.byref(n), 1 if reset else 0))
        return ms.value, n.value

    def fma_peak(self, precision):
        out = ctypes.c_double()
        check(lib().sg_measure_fma_peak(self.h, int(precision), ctypes.byref(out)))
        return out.value

    def fp32_autotune(self, nrhs):
        """(variant, RHS tile, ms best per-receiver tile, ms bucketed, ms best pair-symmetric tile, ms tensor
        cores, ms pair-symmetric tensor cores) for an RHS count; variant -1 if not tuned yet (0 per-receiver,
        1 bucketed, 2 pair-symmetric, 3 pair-symmetric with two warps per receiver, 4 tensor cores,
        5 pair-symmetric tensor cores), a time is -1 when that kernel is not a candidate."""
        v = ctypes.c_int()
        t = ctypes.c_int()
        ms = [ctypes.c_double() for _ in range(5)]
        check(lib().sg_fp32_autotune(self.h, int(nrhs), ctypes.byref(v), ctypes.byref(t),
                                     *[ctypes.byref(m) for m in ms]))
        return (v.value, t.value) + tuple(m.value for m in ms)

    def fp32_set_kernel(self, nrhs, variant, rhs_tile=0):
        """Fix the FP32 operator for an RHS count (0 per-receiver, 1 bucketed, 2 pair-symmetric, 3 pair-symmetric
        with two warps per receiver, 4 tensor cores and 5 pair-symmetric tensor cores with rhs_tile = nrhs)."""
        check(lib().sg_fp32_set_kernel(self.h, int(nrhs), int(variant), int(rhs_tile)))

    def tc_set_window(self, emitters):
        """Emitters per tensor-memory accumulator of the tensor-core operator before it is drained."""
        check(lib().sg_tc_set_window(self.h, int(emitters)))

    # -- learned preconditioner
    def precond_add_graph(self, nbr):
        """Upload a neighbour table nbr[n][k+1] (slot 0 = the particle itself); returns its graph id."""
        nbr = np.ascontiguousarray(nbr, dtype=np.int32)
        gid = ctypes.c_int()
        check(lib().sg_precond_add_graph(self.h, nbr.shape[1] - 1, ptr(nbr), ctypes.byref(gid)))
        return gid.value

    def precond_select(self, graph_id):
        check(lib().sg_precond_select(self.h, int(graph_id)))

    def precond_clear(self):
        check(lib().sg_precond_clear(self.h))

    def precond_set_params(self, blocksize, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        check(lib().sg_precond_set_params(self.h, int(blocksize), ptr(p), p.size))

    def precond_get_params(self, count):
        p = np.zeros(count, np.float32)
        check(lib().sg_precond_get_params(self.h, ptr(p), count))
        return p

    def precond_apply_dev(self, v_ptr, z_ptr, nvec, stream=None):
        check(lib().sg_precond_apply_dev(self.h, ctypes.c_void_p(v_ptr), ctypes.c_void_p(z_ptr), int(nvec),
                                         ctypes.c_void_p(stream or 0)))

    def precond_train_step(self, graph_id, v_ptr, e_ptr, nvec, lr=0.0, step=0, grad=None):
        """Loss of one batch (and the gradient into ``grad`` when given); an Adam step when lr > 0."""
        loss = ctypes.c_double()
        gp = ptr(grad) if grad is not None else None
        check(lib().sg_precond_train_step(self.h, int(graph_id), ctypes.c_void_p(v_ptr), ctypes.c_void_p(e_ptr),
                                          int(nvec), float(lr), int(step), ctypes.byref(loss), gp))
        return loss.value

    def precond_export_blocks(self, graph_id, n, k1, bs):
        out = np.zeros((n, k1, bs, bs), np.complex64)
        check(lib().sg_precond_export_blocks(self.h, int(graph_id), ptr(out)))
        return out

    def bessel_jac_table_dev(self, kappa_ptr, jac_ptr, nk, rho_ptr, nr, nmax, out_ptr, stream=None):
        check(lib().sg_bessel_jac_table(self.h, ctypes.c_void_p(kappa_ptr), ctypes.c_void_p(jac_ptr), int(nk),
                                        ctypes.c_void_p(rho_ptr), int(nr), int(nmax), ctypes.c_void_p(out_ptr),
                                        ctypes.c_void_p(stream or 0)))

    def lookup_contract_dev(self, a_ptr, nr, nk, g_ptr, ncols, cols_ptr, factor, out_ptr, out_stride, stream=None):
        """out[r * out_stride + cols[j]] = factor * sum_k a[r][k] g[k][j] on the device (see the header)."""
        check(lib().sg_lookup_contract(self.h, ctypes.c_void_p(a_ptr), int(nr), int(nk), ctypes.c_void_p(g_ptr),
                                       int(ncols), ctypes.c_void_p(cols_ptr), float(complex(factor).real),
                                       float(complex(factor).imag), ctypes.c_void_p(out_ptr), int(out_stride),
                                       ctypes.c_void_p(stream or 0)))

    def pwe_field_dev(self, field, n, x_ptr, y_ptr, z_ptr, nk, kpar_ptr, kz_ptr, na, alpha_ptr, g_ptr, k, omega,
                      out_ptr, stream=None):
        """Field (0 = E, 1 = H) of a plane-wave expansion at n points (device buffers, see the header)."""
        check(lib().sg_pwe_field(self.h, int(field), int(n), ctypes.c_void_p(x_ptr), ctypes.c_void_p(y_ptr),
                                 ctypes.c_void_p(z_ptr), int(nk), ctypes.c_void_p(kpar_ptr), ctypes.c_void_p(kz_ptr),
                                 int(na), ctypes.c_void_p(alpha_ptr), ctypes.c_void_p(g_ptr), float(np.real(k)),
                                 float(np.imag(k)), float(omega), ctypes.c_void_p(out_ptr),
                                 ctypes.c_void_p(stream or 0)))

    def farfield_sum_dev(self, n, xy_ptr, bs, nrhs, coef_ptr, m_max, m_of_n, nk, kpar_ptr, S_ptr, na, alpha_ptr,
                         out_ptr, stream=None, zphase_ptr=None):
        """Device particle sum of the scattered plane-wave expansion (``zphase_ptr``: per-particle
        height factors [nk][n] for particles at different heights, None when they share one)."""
        mo = np.ascontiguousarray(m_of_n, dtype=np.int32)
        check(lib().sg_farfield_sum_heights(self.h, int(n), ctypes.c_void_p(xy_ptr), int(bs), int(nrhs),
                                            ctypes.c_void_p(coef_ptr), int(m_max), ptr(mo), int(nk),
                                            ctypes.c_void_p(kpar_ptr), ctypes.c_void_p(S_ptr), int(na),
                                            ctypes.c_void_p(alpha_ptr), ctypes.c_void_p(zphase_ptr or 0),
                                            ctypes.c_void_p(out_ptr), ctypes.c_void_p(stream or 0)))

    def plane_wave_swe_dev(self, n_points, xyz_ptr, nwaves, ncomp, kr_ptr, blocksize, amp_ptr, out_ptr, stream=None):
        """Device regular SWE coefficients of plane waves at points (see ``sg_plane_wave_swe``)."""
        check(lib().sg_plane_wave_swe(self.h, int(n_points), ctypes.c_void_p(xyz_ptr), int(nwaves), int(ncomp),
                                      ctypes.c_void_p(kr_ptr), int(blocksize), ctypes.c_void_p(amp_ptr),
                                      ctypes.c_void_p(out_ptr), ctypes.c_void_p(stream or 0)))

    def launch_count(self):
        n = ctypes.c_int64()
        check(lib().sg_launch_count(self.h, ctypes.byref(n)))
        return n.value
