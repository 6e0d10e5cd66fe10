"""Volume lookup (particles at different heights): oracle pinned to the reference, host logic.

The fixture ``vol5`` was made by running the reference's CPU volume lookup
(``CouplingMatrixVolumeLookupCPU``) in the build container (tests/golden/make_golden.py). No GPU.
"""
import numpy as np
import pytest
import scipy.interpolate

import golden_cases as gc
import oracle.physics as ophys
import oracle.solve as osv
import oracle.volume as ovol

VOLUME_CASES = gc.available(volume=True)


@pytest.fixture(scope="module")
def vol5():
    g = gc.load("vol5")
    parts, ls, wl = gc.oracle_inputs(g)
    kp = gc.oracle_contour(g, ls, wl)
    tables = ovol.volumetric_coupling_lookup_table(wl, parts, ls, kp, float(g["resolution"]))
    return g, parts, ls, wl, kp, tables


def test_volume_cases_present():
    assert "vol5" in VOLUME_CASES
    assert "vol5" not in gc.available()


def _check_tables(g, pl, mn, rho, sz, dz):
    np.testing.assert_array_equal(rho, g["rho_grid"])
    np.testing.assert_array_equal(sz, g["sz_grid"])
    np.testing.assert_array_equal(dz, g["dz_grid"])
    for key, t in (("plus", pl), ("minus", mn)):
        assert str(t.dtype) == str(g["table_%s_dtype" % key])
        assert tuple(t.shape) == tuple(g["table_%s_shape" % key])
        # complex64 like the reference: equal entry by entry on the stored rows
        np.testing.assert_array_equal(t[g["table_%s_rows" % key]], g["table_%s_subset" % key])
        tc = t.astype(complex)
        assert abs(np.abs(tc).sum() - g["table_%s_abs_sum" % key]) <= 1e-12 * g["table_%s_abs_sum" % key]
        wts = np.cos(0.37 * np.arange(t.size)).reshape(t.shape)
        assert abs((tc * wts).sum() - g["table_%s_weighted_sum" % key]) <= 1e-10 * np.abs(tc).sum()


def test_oracle_tables_match_reference(vol5):
    g, parts, ls, wl, kp, tables = vol5
    np.testing.assert_array_equal(kp, g["kpar"])
    _check_tables(g, *tables)


def test_oracle_matvec_and_solve_match_reference(vol5):
    g, parts, ls, wl, kp, (pl, mn, rho, sz, dz) = vol5
    T = [ophys.particle_t_matrix(p, wl, ls) for p in parts]
    assert gc.relerr(np.concatenate([np.diag(t) for t in T]), g["t_diag"]) < 1e-14
    _, _, _, offs = osv.system_layout(parts)
    for kind in ("linear", "cubic"):
        W = ovol.VolumeLookupCPU(parts, pl, mn, rho, sz, dz, kind)
        x = g["x_" + kind]
        assert gc.relerr(W.matvec(x), g["Wx_" + kind]) < 1e-14
        assert gc.relerr(osv.master_matvec(W, T, offs, x), g["Mx_" + kind]) < 1e-14
        b, info, _ = osv.gmres_solve(W, T, offs, g["rhs_%s_w0" % kind], 1e-13)
        assert info == 0
        assert gc.relerr(b, g["b_%s_w0" % kind]) < 1e-12


def test_oracle_hermite_is_the_reference_cuda_formula(vol5):
    """Catmull-Rom taps reproduce grid values at nodes and linear data exactly (the reference CUDA
    kernel's cubic_interpolation is exact for quadratics)."""
    w = np.linspace(0, 1, 7)
    for p in (lambda t: 1 + 0 * t, lambda t: t, lambda t: t * t):
        taps = np.array([p(-1.0), p(0.0), p(1.0), p(2.0)])
        np.testing.assert_allclose(ovol._catmull_rom(w).T @ taps, p(w), atol=1e-14)
    g, parts, ls, wl, kp, (pl, mn, rho, sz, dz) = vol5
    Wh = ovol.VolumeLookupCPU(parts, pl, mn, rho, sz, dz, "cubic_hermite")
    Ws = ovol.VolumeLookupCPU(parts, pl, mn, rho, sz, dz, "cubic")
    x = g["x_cubic"]
    # both are cubic interpolants of the same table: close, not equal
    assert 0 < gc.relerr(Wh.matvec(x), Ws.matvec(x)) < 1e-2


def test_moment_form_spline_equals_rect_bivariate_spline():
    """The GPU kernel's tensor-product spline (values + h^2 node moments) is RectBivariateSpline(3, 3)."""
    rng = np.random.default_rng(0)
    for nx, ny in ((12, 9), (5, 4), (4, 7)):
        f = rng.standard_normal((nx, ny)) + 1j * rng.standard_normal((nx, ny))
        h = 0.7
        xg = -2.1 + h * np.arange(nx)
        yg = 1.3 + h * np.arange(ny)
        mx = ovol.spline_moments(f, 0)
        my = ovol.spline_moments(f, 1)
        mxy = ovol.spline_moments(mx, 1)
        sr = scipy.interpolate.RectBivariateSpline(xg, yg, f.real, kx=3, ky=3)
        si = scipy.interpolate.RectBivariateSpline(xg, yg, f.imag, kx=3, ky=3)
        for _ in range(50):
            x = rng.uniform(xg[0], xg[-1] - 1e-9)
            y = rng.uniform(yg[0], yg[-1] - 1e-9)
            ia, ib = int((x - xg[0]) // h), int((y - yg[0]) // h)
            ia, ib = min(ia, nx - 2), min(ib, ny - 2)
            v = ovol.moment_spline_eval(f, mx, my, mxy, ia, (x - xg[ia]) / h, ib, (y - yg[ib]) / h)
            assert abs(v - (sr.ev(x, y) + 1j * si.ev(x, y))) < 1e-12 * (1 + np.abs(f).max())


def _product_inputs(g):
    from smuthi_gb300 import layers, particles
    parts = [particles.Sphere(position=list(p), refractive_index=complex(n), radius=float(r), l_max=int(lm),
                              m_max=int(mm))
             for p, n, r, lm, mm in zip(g["positions"], g["n_particle"], g["radii"], g["l_max"], g["m_max"])]
    ls = layers.LayerSystem([float(x) for x in g["thicknesses"]], [complex(x) for x in g["layer_n"]])
    return parts, ls, float(g["wavelength"])


def test_product_table_builder_matches_reference():
    """Host part of the product's table build (Bessel factors on the host here) is bit-equal to the
    reference's complex64 tables."""
    from smuthi_gb300.linearsystem.particlecoupling import prepare_lookup as look
    g = gc.load("vol5")
    parts, ls, wl = _product_inputs(g)
    _check_tables(g, *look.volumetric_coupling_lookup_table(wl, parts, ls, g["kpar"], float(g["resolution"])))


def test_product_cross_sections_host_path():
    """Cross sections of particles at different heights with mixed cut-offs (host particle sum)."""
    from smuthi_gb300 import fields as flds
    from smuthi_gb300 import initial_field as init
    from smuthi_gb300.postprocessing import far_field as ff
    g = gc.load("vol5")
    parts, ls, wl = _product_inputs(g)
    offs = np.concatenate([[0], np.cumsum([flds.blocksize(p.l_max, p.m_max) for p in parts])])
    for tag in ("linear_w0", "linear_w1", "cubic_w0"):
        pw = gc.plane_wave(g, int(tag.split("_w")[1]), init.PlaneWave)
        b = g["b_" + tag]
        coefs = [b[offs[i]:offs[i + 1]] for i in range(len(parts))]
        ext = ff.extinction_cross_section(initial_field=pw, particle_list=parts, layer_system=ls, coefficients=coefs)
        sca = ff.total_scattering_cross_section(initial_field=pw, particle_list=parts, layer_system=ls,
                                                coefficients=coefs)
        assert abs(ext - g["sigma_ext_" + tag]) <= 1e-12 * abs(g["sigma_ext_" + tag])
        assert abs(sca - g["sigma_sca_" + tag]) <= 1e-12 * abs(g["sigma_sca_" + tag])
