"""The allocation-free coupling matvec agrees with the reference's W x and the context-based one.

sg_coupling_matvec_linear_noalloc serves callers that cannot allocate device memory while they
compute (their device memory belongs to another framework's pool, or their budget is fixed after
start-up): it takes caller-owned device buffers and keeps its scratch in a static device array.
This file is collected last so that a run stopping at the first failure has already run every
other test; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu


def _setup():
    import torch
    from smuthi_gb300 import _lib, layers, particles
    from smuthi_gb300.build import build
    from smuthi_gb300.linearsystem import linear_system as lsm
    build()
    g = gc.load("c1")
    parts = [particles.Sphere(position=list(p), refractive_index=complex(n), radius=float(r), l_max=int(lm),
                              m_max=int(mm))
             for p, n, r, lm, mm in zip(g["positions"], g["n_particle"], g["radii"], g["l_max"], g["m_max"])]
    ls = layers.LayerSystem([float(x) for x in g["thicknesses"]], [float(complex(x).real) for x in g["layer_n"]])
    ctx = _lib.Context(0)
    W = lsm.CouplingMatrixRadialLookupCUDA(float(g["wavelength"]), parts, ls, k_parallel=g["kpar"],
                                           resolution=float(g["resolution"]), interpolator_kind="linear",
                                           context=ctx)
    torch.cuda.set_device(0)
    return torch, _lib, g, ctx, W


def _noalloc(_lib, g, W, xy, mofn, table, x, y, nrhs, stream):
    n, bs = len(g["positions"]), W.blocksize
    return _lib.lib().sg_coupling_matvec_linear_noalloc(
        0, n, ctypes.c_void_p(xy.data_ptr()), bs, ctypes.c_void_p(mofn.data_ptr()), table.shape[0],
        float(W.radial_distance_array[0]), float(g["resolution"]), ctypes.c_void_p(table.data_ptr()),
        ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), nrhs, ctypes.c_void_p(stream))


def test_noalloc_matches_context_matvec_twice():
    torch, _lib, g, ctx, W = _setup()
    dev = torch.device("cuda", 0)
    n, bs = len(g["positions"]), W.blocksize
    xy = torch.from_numpy(np.ascontiguousarray(g["positions"][:, :2])).to(dev)
    mofn = torch.from_numpy(W.m_of_n.astype(np.int32)).to(dev)
    table = torch.from_numpy(np.ascontiguousarray(W.lookup_table)).to(dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    # the reference's own W x of the fixture (linear lookup), two calls in a row
    x0 = torch.from_numpy(np.ascontiguousarray(g["x_linear"][:, None])).to(dev)
    for _ in range(2):
        y0 = torch.full_like(x0, float("nan"))
        _lib.check(_noalloc(_lib, g, W, xy, mofn, table, x0, y0, 1, stream))
        torch.cuda.synchronize(dev)
        assert gc.relerr(y0.cpu().numpy()[:, 0], g["Wx_linear"]) < 1e-12
    # after the first call on the device a warmed entry point allocates no device memory
    rng = np.random.default_rng(11)
    for nrhs in (1, 3):
        X = rng.standard_normal((n * bs, nrhs)) + 1j * rng.standard_normal((n * bs, nrhs))
        x = torch.from_numpy(np.ascontiguousarray(X)).to(dev)
        y_ref = torch.empty_like(x)
        ctx.coupling_matvec_dev(x.data_ptr(), y_ref.data_ptr(), nrhs, _lib.SG_FP64, stream=stream)
        y = torch.full_like(x, float("nan"))
        torch.cuda.synchronize(dev)
        free1 = torch.cuda.mem_get_info(dev)[0]
        for _ in range(2):  # two calls in a row share (and overwrite) the static scratch
            y.fill_(float("nan"))
            _lib.check(_noalloc(_lib, g, W, xy, mofn, table, x, y, nrhs, stream))
            torch.cuda.synchronize(dev)
            assert torch.cuda.mem_get_info(dev)[0] == free1
            assert gc.relerr(y.cpu().numpy(), y_ref.cpu().numpy()) < 1e-12
    ctx.close()


def test_noalloc_rejects_too_many_rhs():
    torch, _lib, g, ctx, W = _setup()
    rc = _lib.lib().sg_coupling_matvec_linear_noalloc(0, 1, ctypes.c_void_p(8), 2, ctypes.c_void_p(8), 10, -15.0,
                                                      5.0, ctypes.c_void_p(8), ctypes.c_void_p(8),
                                                      ctypes.c_void_p(8), 65536, None)
    assert rc == _lib.SG_ERR_ARG
    assert b"65535" in _lib.lib().sg_last_error()
    ctx.close()


def test_noalloc_rejects_sizes_beyond_scratch():
    torch, _lib, g, ctx, W = _setup()
    n, bs = len(g["positions"]), W.blocksize
    nrhs = (1 << 20) // (n * bs) + 1  # one RHS more than the 16 MiB scratch holds
    rc = _lib.lib().sg_coupling_matvec_linear_noalloc(0, n, ctypes.c_void_p(8), bs, ctypes.c_void_p(8), 10, -15.0,
                                                      5.0, ctypes.c_void_p(8), ctypes.c_void_p(8),
                                                      ctypes.c_void_p(8), nrhs, None)
    assert rc == _lib.SG_ERR_ARG
    assert b"static" in _lib.lib().sg_last_error()
    ctx.close()
