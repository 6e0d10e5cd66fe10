"""Every FP32 operator kernel against the FP64 operator and the reference's own outputs.

The FP32 operator drives the correction solves of the mixed-precision refinement; the autotuner
picks among the per-receiver kernel (RHS tiles 1-16), the interval-bucketed kernel and the
pair-symmetric kernel (one interpolation per unordered pair for both directions, with one or two warps
per receiver). The tensor-core operators (variant 4: tcgen05 3xTF32 with drained
accumulators; variant 5: the same with one interpolated block per unordered pair) are held to the same bound. Each is fixed
here with ``fp32_set_kernel`` and compared, through the C ABI, with the FP64 operator (relative
2-norm 2e-5, the FP32 bound the other FP32 tests use) and with the reference's W x / M x.
Also: the full (non-diagonal) T-matrix epilogue of the FP64, per-receiver FP32 and pair-symmetric
kernels against x - T (W x) formed on the host from the FP64 W x.
"""
import numpy as np
import pytest

import golden_cases as gc
from test_gpu_parity import _kinds, _product_system

pytestmark = pytest.mark.gpu

TOL32 = 2e-5


def _variants(ctx, R, bs):
    """(variant, tile) pairs the library accepts for R right-hand sides."""
    out = [(0, t) for t in (1, 2, 4, 8, 16) if R % t == 0]
    out += [(2, t) for t in (1, 2, 4, 8, 16) if R % t == 0 and t <= (16 if bs <= 32 else 8)]
    out += [(3, t) for t in (4, 8, 16) if R % t == 0 and t <= (16 if bs <= 32 else 8)]
    if R in (16, 32, 64) and bs <= 48:
        out.append((4, R))
    if R in (16, 32) and bs <= 32:
        out.append((5, R))
    return out


def _rhs(x, R, seed):
    if R == 1:
        return x
    rng = np.random.default_rng(seed)
    cols = [x] + [x * (1 + 0.5 * rng.standard_normal(x.shape)) + 0.2j * rng.standard_normal(x.shape)
                  for _ in range(R - 1)]
    return np.ascontiguousarray(np.stack(cols, axis=1))


@pytest.mark.parametrize("name", gc.available())
def test_fp32_kernels_match_fp64_and_reference(name, gpu_context):
    from smuthi_gb300 import _lib
    g = gc.load(name)
    for kind in _kinds(g):
        parts, ls, wl, W, M = _product_system(g, kind, gpu_context)
        bs = int(max((p.l_max * (p.l_max + 2) * 2) for p in parts))  # upper bound of the padded blocksize
        x = g["x_" + kind]
        for R in (1, 3, 16, 64):
            X = _rhs(x, R, 7)
            y64 = gpu_context.coupling_matvec(X, _lib.SG_FP64)
            m64 = gpu_context.master_matvec(X, _lib.SG_FP64)
            # the double-float operator at the RHS tile its autotuner picks for R (4, 8 or 16)
            assert gc.relerr(gpu_context.master_matvec(X, _lib.SG_DF64), m64) < 1e-12, (name, kind, R)
            for v, t in _variants(gpu_context, R, bs):
                gpu_context.fp32_set_kernel(R, v, t)
                y32 = gpu_context.coupling_matvec(X, _lib.SG_FP32)
                m32 = gpu_context.master_matvec(X, _lib.SG_FP32)
                assert gc.relerr(y32, y64) < TOL32, (name, kind, R, v, t)
                assert gc.relerr(m32, m64) < TOL32, (name, kind, R, v, t)
                col0 = y32 if R == 1 else y32[:, 0]
                assert gc.relerr(col0, g["Wx_" + kind]) < TOL32, (name, kind, R, v, t)


@pytest.mark.parametrize("name", ["c5s", "c3s"])
def test_full_t_epilogue(name, gpu_context):
    """Dense T blocks (two particle types): every kernel's fused x - T W x against the host."""
    from smuthi_gb300 import _lib
    g = gc.load(name)
    kind = _kinds(g)[0]
    parts, ls, wl, W, M = _product_system(g, kind, gpu_context)
    n = len(parts)
    bs = W.shape[0] // n
    rng = np.random.default_rng(11)
    blocks = 0.05 * (rng.standard_normal((2, bs, bs)) + 1j * rng.standard_normal((2, bs, bs)))
    types = (np.arange(n) % 2).astype(np.int32)
    gpu_context.set_tmatrix(blocks, types, diagonal=False)
    for R in (1, 4, 16):
        X = _rhs(g["x_" + kind], R, 3)
        Xr = X.reshape(n, bs, R)
        wx = gpu_context.coupling_matvec(X, _lib.SG_FP64).reshape(n, bs, R)
        ref = (Xr - np.einsum("iab,ibr->iar", blocks[types], wx)).reshape(X.shape)
        assert gc.relerr(gpu_context.master_matvec(X, _lib.SG_FP64), ref) < 1e-13
        tensor = [(4, 16)] + ([(5, 16)] if bs <= 32 else [])
        for v, t in [(0, 1), (2, 1)] + ([(0, 4), (2, 4), (3, 4)] if R == 4 else []) + (tensor if R == 16 else []):
            gpu_context.fp32_set_kernel(R, v, t)
            assert gc.relerr(gpu_context.master_matvec(X, _lib.SG_FP32), ref) < TOL32, (R, v, t)


def test_fp32_set_kernel_rejects_bad_choices(gpu_context):
    from smuthi_gb300 import _lib
    g = gc.load("c1")
    _product_system(g, "linear", gpu_context)
    for args in [(16, 0, 3), (4, 0, 8), (16, 2, 32), (6, 2, 4), (4, 6, 1), (2, 3, 2), (8, 4, 8), (16, 4, 8), (64, 5, 64),
                 (16, 5, 8)]:
        with pytest.raises(_lib.SmuthiGB300Error) as e:
            gpu_context.fp32_set_kernel(*args)
        assert e.value.code == _lib.SG_ERR_ARG


def test_full_size_c2_symmetric_kernel(gpu_context):
    """2000 spheres (cubic, 16 RHS): the pair-symmetric kernel against the per-receiver FP32 kernel and
    the FP64 operator, and the autotuner's report of all three FP32 kernels."""
    from smuthi_gb300 import _lib, layers, particles, workloads
    import smuthi_gb300.fields as flds
    from smuthi_gb300.linearsystem import linear_system as lsm
    spec = workloads.build("c2", seed=0)
    parts = [particles.Sphere(position=list(p), refractive_index=spec["n_particle"], radius=spec["radius"],
                              l_max=3, m_max=3) for p in spec["positions"]]
    ls = layers.LayerSystem(*spec["layers"])
    wl = spec["wavelength"]
    kp = flds.reasonable_Sommerfeld_kpar_contour(wl, layer_refractive_indices=ls.refractive_indices)
    W = lsm.CouplingMatrixRadialLookupCUDA(wl, parts, ls, k_parallel=kp, resolution=spec["resolution"],
                                           interpolator_kind="cubic", context=gpu_context)
    rng = np.random.default_rng(9)
    X = np.ascontiguousarray(rng.standard_normal((W.shape[0], 16)) + 1j * rng.standard_normal((W.shape[0], 16)))
    y64 = gpu_context.coupling_matvec(X, _lib.SG_FP64)
    assert gc.relerr(gpu_context.coupling_matvec(X, _lib.SG_DF64), y64) < 1e-12
    gpu_context.fp32_set_kernel(16, 2, 16)
    ys = gpu_context.coupling_matvec(X, _lib.SG_FP32)
    gpu_context.fp32_set_kernel(16, 3, 16)
    assert gc.relerr(gpu_context.coupling_matvec(X, _lib.SG_FP32), y64) < TOL32
    for v in (4, 5):
        gpu_context.fp32_set_kernel(16, v, 16)
        assert gc.relerr(gpu_context.coupling_matvec(X, _lib.SG_FP32), y64) < 5e-6, v
    gpu_context.fp32_set_kernel(16, 0, 8)
    yr = gpu_context.coupling_matvec(X, _lib.SG_FP32)
    assert gc.relerr(ys, y64) < TOL32
    assert gc.relerr(yr, y64) < TOL32
    # the autotuner times all candidates again after a new lookup
    W2 = lsm.CouplingMatrixRadialLookupCUDA(wl, parts, ls, k_parallel=kp, resolution=spec["resolution"],
                                            interpolator_kind="cubic", context=gpu_context)
    yt = gpu_context.coupling_matvec(X, _lib.SG_FP32)
    assert gc.relerr(yt, y64) < TOL32
    variant, tile, ms_rec, ms_bucket, ms_sym, ms_tc, ms_tcs = gpu_context.fp32_autotune(16)
    assert variant in (0, 1, 2, 3, 4, 5) and ms_rec > 0 and ms_sym > 0 and ms_tc > 0 and ms_tcs > 0
    del W2


def test_full_size_c3_operator_and_mixed_solve(gpu_context):
    """5000 spheres, blocksize 48, cubic lookup at 2 nm (the mixed-precision shape at full size): FP64
    operator rows against the oracle, every FP32 kernel against FP64 at 4 RHS, the tensor-core operator
    against the double-float operator at 64 RHS (bound 5e-6), and the chosen form's solve of 64 plane
    waves (the 64-wave batch of this shape) to an FP64-grade relative residual of 1e-6, re-checked with
    the FP64 operator on four of the waves."""
    import oracle.physics as ophys
    import oracle.solve as osv
    from smuthi_gb300 import _lib, learned
    system = learned.film_system("c3", nrhs=64, ctx=gpu_context)
    W, n, bs = system["W"], system["n"], system["blocksize"]
    assert (n, bs) == (5000, 48)
    rng = np.random.default_rng(13)
    x = rng.standard_normal(W.shape[0]) + 1j * rng.standard_normal(W.shape[0])
    y = gpu_context.coupling_matvec(x, _lib.SG_FP64)
    rows = np.array([0, 2500, 4999])
    oparts = [ophys.Sphere(p.position, p.refractive_index, p.radius, p.l_max, p.m_max) for p in system["parts"]]
    Wo = osv.RadialLookupCPU(oparts, W.lookup_table, W.radial_distance_array, "cubic")
    yo = Wo.matvec(x, rows=rows)
    sel = np.concatenate([np.arange(r * bs, (r + 1) * bs) for r in rows])
    assert gc.relerr(y[sel], yo[sel]) < 1e-11
    B = np.ascontiguousarray(system["rhs"])
    X4 = np.ascontiguousarray(B[:, :4])
    y64 = gpu_context.coupling_matvec(X4, _lib.SG_FP64)
    for v, t in [(0, 4), (2, 4), (3, 4)]:
        gpu_context.fp32_set_kernel(4, v, t)
        assert gc.relerr(gpu_context.coupling_matvec(X4, _lib.SG_FP32), y64) < TOL32, (v, t)
    ydf = gpu_context.coupling_matvec(B, _lib.SG_DF64)
    assert gc.relerr(ydf[:, :4], y64) < 1e-12
    assert gc.relerr(gpu_context.coupling_matvec(B, _lib.SG_TF32X3), ydf) < 5e-6
    sol, info = gpu_context.gmres(B, np.zeros_like(B), 1e-6, restart=64, precision=_lib.SG_FP32 | _lib.SG_DF64)
    assert info.converged == 64
    assert gpu_context.true_residual(X4, np.ascontiguousarray(sol[:, :4])).max() <= 1e-6
