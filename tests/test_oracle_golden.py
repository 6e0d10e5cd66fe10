"""The oracle reproduces the reference's own outputs (golden fixtures made by running it)."""
import numpy as np
import pytest

import golden_cases as gc
import oracle.crosssections as ocs
import oracle.physics as ophys
import oracle.solve as osv

CASES = gc.available()


@pytest.fixture(scope="module", params=CASES)
def case(request):
    g = gc.load(request.param)
    parts, ls, wl = gc.oracle_inputs(g)
    kp = gc.oracle_contour(g, ls, wl)
    return request.param, g, parts, ls, wl, kp


def test_contour_and_table(case):
    name, g, parts, ls, wl, kp = case
    np.testing.assert_array_equal(kp, g["kpar"])
    tab, rho = ophys.radial_coupling_lookup_table(wl, parts, ls, kp, float(g["resolution"]))
    np.testing.assert_array_equal(rho, g["rho_grid"])
    assert tuple(tab.shape) == tuple(g["table_shape"])
    if "table" in g:
        assert gc.relerr(tab, g["table"]) < 1e-14
    else:
        assert gc.relerr(tab[g["table_rows"]], g["table_subset"]) < 1e-14
    assert abs(np.abs(tab).sum() - g["table_abs_sum"]) <= 1e-12 * g["table_abs_sum"]
    wts = np.cos(0.37 * np.arange(tab.size)).reshape(tab.shape)
    assert abs((tab * wts).sum() - g["table_weighted_sum"]) <= 1e-10 * np.abs(tab).sum()


def test_tmatrix_rhs(case):
    name, g, parts, ls, wl, kp = case
    T = [ophys.particle_t_matrix(p, wl, ls) for p in parts]
    assert gc.relerr(np.concatenate([np.diag(t) for t in T]), g["t_diag"]) < 1e-14
    _, _, _, offs = osv.system_layout(parts)
    for key in [k for k in g if k.startswith("a_")]:
        tag = key[2:]
        pw = gc.plane_wave(g, int(tag.split("_w")[1]))
        a = [ophys.initial_field_coefficients(pw, p, ls) for p in parts]
        assert gc.relerr(np.concatenate(a), g[key]) < 1e-14
        assert gc.relerr(osv.right_hand_side(T, offs, a), g["rhs_" + tag]) < 1e-14


def test_cross_sections_from_reference_solution(case):
    name, g, parts, ls, wl, kp = case
    _, _, _, offs = osv.system_layout(parts)
    if name not in ("wg3", "c5s"):
        pytest.skip("cross-section oracle timing: checked on the small cases")
    for key in [k for k in g if k.startswith("b_")]:
        tag = key[2:]
        pw = gc.plane_wave(g, int(tag.split("_w")[1]))
        b = g[key]
        coefs = [b[offs[i]:offs[i + 1]] for i in range(len(parts))]
        ext = ocs.extinction_cross_section(pw, parts, coefs, ls)
        assert abs(ext - g["sigma_ext_" + tag]) <= 1e-12 * abs(g["sigma_ext_" + tag])
        if name == "wg3":
            sca = ocs.total_scattering_cross_section(pw, parts, coefs, ls)
            assert abs(sca - g["sigma_sca_" + tag]) <= 1e-12 * abs(g["sigma_sca_" + tag])


def test_matvec_and_solve_small():
    g = gc.load("wg3")
    parts, ls, wl = gc.oracle_inputs(g)
    kp = gc.oracle_contour(g, ls, wl)
    tab, rho = ophys.radial_coupling_lookup_table(wl, parts, ls, kp, float(g["resolution"]))
    T = [ophys.particle_t_matrix(p, wl, ls) for p in parts]
    _, _, _, offs = osv.system_layout(parts)
    for kind in ("linear", "cubic"):
        W = osv.RadialLookupCPU(parts, tab, rho, kind)
        x = g["x_" + kind]
        assert gc.relerr(W.matvec(x), g["Wx_" + kind]) < 1e-14
        assert gc.relerr(osv.master_matvec(W, T, offs, x), g["Mx_" + kind]) < 1e-14
        b, info, _ = osv.gmres_solve(W, T, offs, g["rhs_%s_w0" % kind], 1e-13)
        assert info == 0
        assert gc.relerr(b, g["b_%s_w0" % kind]) < 1e-12
