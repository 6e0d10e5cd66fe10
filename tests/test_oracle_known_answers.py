"""Pin the oracle against the known-answer values hard-coded in the reference's own tests."""
import numpy as np
import pytest

import oracle.layers as olay
import oracle.physics as ophys
import oracle.special as osp


def test_mie_against_prototype():
    # tests/unit_tests/t_matrix_tests/test_t_matrix.py:11-27
    omega = 2 * 3.15 / 550
    n_medium, n_particle, radius, l = 1.6 + 0.1j, 2.6 + 0.4j, 260, 4
    q0 = ophys.mie_coefficient(0, l, omega * n_medium, omega * n_particle, radius)
    q1 = ophys.mie_coefficient(1, l, omega * n_medium, omega * n_particle, radius)
    np.testing.assert_almost_equal(q0, -0.421469104177215 - 0.346698396584972j)
    np.testing.assert_almost_equal(q1, -0.511272170262304 - 0.061284547954858j)


def test_layer_response_against_prototype():
    # tests/unit_tests/test_layerresponse.py:10-14, 40-53
    layer_d = [0, 300, 400, 0]
    layer_n = [1, 2 + 0.1j, 3, 1 + 5j]
    omega = 2 * 3.15 / 550
    kpar = omega * 1.7
    l1 = olay.response_matrix_scalar(0, layer_d, layer_n, kpar, omega, 2, 1)
    np.testing.assert_almost_equal(l1, np.array([[-0.392979481352895 - 0.376963315605839j,
                                                  -0.455367266697897 + 0.426065579868901j],
                                                 [0.545168303416962 - 0.345873455516963j,
                                                  -0.361796569025878 - 0.644799225334747j]]))
    l2 = olay.response_matrix_scalar(1, layer_d, layer_n, kpar, omega, 1, 2)
    np.testing.assert_almost_equal(l2, np.array([[-0.240373686730040 - 0.148769054113797j,
                                                  0.161922209423045 + 0.222085165907288j],
                                                 [-0.182951011363592 + 0.138158890222525j,
                                                  0.215395950986834 - 0.057346289106977j]]))


def test_scattering_matrix_equals_transfer_matrix():
    # tests/unit_tests/test_layerresponse.py:30-36
    layer_d = [0, 300, 400, 0]
    layer_n = [1, 2 + 0.1j, 3, 1 + 5j]
    omega = 2 * 3.15 / 550
    kpar = omega * 1.7
    for pol in (0, 1):
        t = olay.transfer_matrix(pol, layer_d, layer_n, kpar, omega)
        s = olay.scattering_matrix(pol, layer_d, layer_n, kpar, omega)
        np.testing.assert_almost_equal(t[1, 0] / t[0, 0], s[1, 0])


def test_legendre_against_prototype():
    # tests/unit_tests/vwf_and_transformations_tests/test_spherical_functions.py:20-46
    omega = 2 * 3.14 / 550
    kp = omega * np.array([0.01, 0.2, 0.7, 0.99, 1.2, 2 - 0.5j])
    kz = np.sqrt(omega ** 2 - kp ** 2 + 0j)
    kz[kz.imag < 0] = -kz[kz.imag < 0]
    plm, _, _ = osp.legendre_normalized(kz / omega, kp / omega, 3)
    np.testing.assert_almost_equal(plm[3, 0], [1.870267465826245, 1.649727250184103, -0.300608757357466,
                                               -0.382739631607606, -3.226515147957620j,
                                               -25.338383323084539 - 22.141864985871653j])
    np.testing.assert_almost_equal(plm[2, 1], [0.019363948460993, 0.379473319220206, 0.968052168015753,
                                               0.270444009917026, 1.541427909439815j,
                                               3.906499971729346 + 6.239600710712296j])


def test_wigner3j_against_sympy():
    sympy_w = pytest.importorskip("sympy.physics.wigner")
    for args in [(1, 1, 0, 0, 0, 0), (2, 3, 4, 1, -1, 0), (3, 3, 2, 2, -1, -1), (4, 4, 8, 4, -4, 0),
                 (2, 1, 3, -2, 1, 1), (3, 2, 0, 0, 0, 0), (4, 3, 5, -3, 2, 1), (2, 2, -1, 0, 0, 0)]:
        ref = float(sympy_w.wigner_3j(*args)) if args[2] >= 0 else 0.0
        assert abs(osp.wigner3j(*args) - ref) <= 1e-15 * max(1.0, abs(ref))


def test_index_map_matches_reference_table():
    # smuthi/fields/__init__.py:34-60 (first rows of the documented index table)
    assert osp.multi_to_single_index(0, 1, -1, 3, 3) == 0
    assert osp.multi_to_single_index(0, 1, 0, 3, 3) == 1
    assert osp.multi_to_single_index(0, 2, -2, 3, 3) == 3
    assert osp.blocksize(3, 3) == 30
    assert osp.blocksize(4, 4) == 48
    assert osp.blocksize(3, 2) == 26
