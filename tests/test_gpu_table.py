"""GPU Bessel factors of the layer-mediated lookup table against scipy and the reference's tables.

The CUDA coupling class builds the layer-mediated part of its table with the library's Bessel
kernel (series / Miller recurrence / Hankel asymptotics) instead of scipy.special.jv; the values
must agree with scipy to 1e-12 of the largest value per order, and whole tables with the host build
and with the reference's own table rows to 1e-12 (relative 2-norm).
"""
import numpy as np
import pytest
import scipy.special

import golden_cases as gc

pytestmark = pytest.mark.gpu


def _bessel_gpu(ctx, kp, jac, rho, nmax):
    import torch
    dev = torch.device("cuda", 0)
    kp_d = torch.from_numpy(np.ascontiguousarray(kp, np.complex128)).to(dev)
    jac_d = torch.from_numpy(np.ascontiguousarray(jac, np.complex128)).to(dev)
    rho_d = torch.from_numpy(np.ascontiguousarray(rho, np.float64)).to(dev)
    out = torch.empty((nmax + 1, len(rho), len(kp)), dtype=torch.complex128, device=dev)
    ctx.bessel_jac_table_dev(kp_d.data_ptr(), jac_d.data_ptr(), len(kp), rho_d.data_ptr(), len(rho), nmax,
                             out.data_ptr())
    torch.cuda.synchronize(dev)
    return out.cpu().numpy()


@pytest.mark.parametrize("shape", ["c2", "c5"])
def test_bessel_factors_match_scipy(gpu_context, shape):
    from smuthi_gb300 import fields as flds, layers, workloads
    spec = workloads.SHAPES[shape]
    ls = layers.LayerSystem(*spec["layers"])
    kp = np.asarray(flds.reasonable_Sommerfeld_kpar_contour(spec["wavelength"],
                                                            layer_refractive_indices=ls.refractive_indices))
    # radial grid points across the whole range of the shape (series, Miller, asymptotic regimes),
    # including the negative start of the grid and rho = 0
    rmax = spec["side"] * np.sqrt(2)
    rho = np.concatenate([np.arange(-15.0, 40.0, 5.0), np.linspace(40.0, rmax, 397)])
    jac = np.exp(1j * np.linspace(0, 3, len(kp))) * (1 + np.arange(len(kp)) / len(kp))
    nmax = 8
    got = _bessel_gpu(gpu_context, kp, jac, rho, nmax)
    for n in range(nmax + 1):
        ref = scipy.special.jv(n, kp[None, :] * rho[:, None]) * jac[None, :]
        err = np.abs(got[n] - ref)
        assert err.max() <= 1e-12 * np.abs(ref).max(), (n, err.max(), np.abs(ref).max())


@pytest.mark.parametrize("name", gc.available())
def test_gpu_built_table_matches_host_and_reference(gpu_context, name):
    from smuthi_gb300 import layers, particles
    from smuthi_gb300.linearsystem.particlecoupling import prepare_lookup as look
    g = gc.load(name)
    parts = [particles.Sphere(position=list(p), refractive_index=complex(n), radius=float(r), l_max=int(lm),
                              m_max=int(mm))
             for p, n, r, lm, mm in zip(g["positions"], g["n_particle"], g["radii"], g["l_max"], g["m_max"])]
    ln = [complex(x) if complex(x).imag else float(complex(x).real) for x in g["layer_n"]]
    ls = layers.LayerSystem([float(x) for x in g["thicknesses"]], ln)
    kw = dict(vacuum_wavelength=float(g["wavelength"]), particle_list=parts, layer_system=ls,
              k_parallel=g["kpar"], resolution=float(g["resolution"]))
    host, rho_h = look.radial_coupling_lookup_table(**kw)
    gpu, rho_g = look.radial_coupling_lookup_table(context=gpu_context, **kw)
    assert np.array_equal(rho_h, rho_g)
    assert gc.relerr(gpu, host) < 1e-12, gc.relerr(gpu, host)
    if "table" in g:
        assert gc.relerr(gpu, g["table"]) < 1e-12
    else:
        rows = g["table_rows"]
        assert gc.relerr(gpu[rows], g["table_subset"]) < 1e-12


def test_bessel_argument_checks(gpu_context):
    from smuthi_gb300 import _lib
    with pytest.raises(_lib.SmuthiGB300Error):
        gpu_context.bessel_jac_table_dev(8, 8, 1, 8, 1, 33, 8)  # order beyond the kernel's table
    with pytest.raises(_lib.SmuthiGB300Error):
        gpu_context.bessel_jac_table_dev(8, 8, 0, 8, 1, 4, 8)  # empty contour


def test_contraction_kernel_matches_numpy(gpu_context):
    """sg_lookup_contract on ragged sizes (rows, contour points and columns not multiples of its tiles)
    with scattered output columns, against numpy in FP64; columns not listed stay untouched."""
    import torch
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(4)
    nr, nk, nc, stride = 131, 37, 45, 60
    a = rng.standard_normal((nr, nk)) + 1j * rng.standard_normal((nr, nk))
    g = rng.standard_normal((nk, nc)) + 1j * rng.standard_normal((nk, nc))
    cols = rng.permutation(stride)[:nc].astype(np.int32)
    fac = 2 * 1j ** 3
    out = np.full((nr, stride), 7.0 + 0j)
    a_d, g_d, c_d = (torch.from_numpy(np.ascontiguousarray(v)).to(dev) for v in (a, g, cols))
    o_d = torch.from_numpy(out.copy()).to(dev)
    gpu_context.lookup_contract_dev(a_d.data_ptr(), nr, nk, g_d.data_ptr(), nc, c_d.data_ptr(), fac, o_d.data_ptr(),
                                    stride)
    torch.cuda.synchronize(dev)
    got = o_d.cpu().numpy()
    ref = out.copy()
    ref[:, cols] = fac * (a @ g)
    assert gc.relerr(got, ref) < 1e-14
    from smuthi_gb300 import _lib
    with pytest.raises(_lib.SmuthiGB300Error):
        gpu_context.lookup_contract_dev(a_d.data_ptr(), nr, nk, g_d.data_ptr(), 0, c_d.data_ptr(), fac,
                                        o_d.data_ptr(), stride)
