"""Near-field evaluation of plane-wave expansions: oracle pinned to the reference, host logic. No GPU.

Fixtures: ``pwe1`` (seeded expansions of both kinds on a complex contour, fields evaluated by the
reference's CPU code in double precision) and ``vol5`` (the scattered field of the reference's
solution above the particles, from its own scattered_field_pwe).
"""
import numpy as np

import golden_cases as gc
import oracle.nearfield as onf


def _oracle_pwe(g, kind):
    lo, hi = g["bounds_" + kind]
    p = onf.PlaneWaveExpansion(complex(g["k"]), g["kpar"], g["alpha"], kind, list(g["ref_" + kind]), lo, hi)
    p.coefficients = g["g_" + kind]
    return p


def test_oracle_fields_match_reference():
    g = gc.load("pwe1")
    pts = g["points"]
    for kind in ("upgoing", "downgoing"):
        p = _oracle_pwe(g, kind)
        E = np.array(p.field(pts[:, 0], pts[:, 1], pts[:, 2], 'E'))
        H = np.array(p.field(pts[:, 0], pts[:, 1], pts[:, 2], 'H', float(g["wavelength"])))
        assert gc.relerr(E, g["E_" + kind]) < 1e-13
        assert gc.relerr(H, g["H_" + kind]) < 1e-13
        # points outside the validity range give exactly zero
        outside = ~p.valid(pts[:, 0], pts[:, 1], pts[:, 2])
        assert outside.any()
        assert np.all(g["E_" + kind][:, outside] == 0) and np.all(E[:, outside] == 0)


def _vol5_particles(g):
    from smuthi_gb300 import fields as flds
    from smuthi_gb300 import layers, particles
    from smuthi_gb300.fields.expansions import SphericalWaveExpansion
    parts = [particles.Sphere(position=list(p), refractive_index=complex(n), radius=float(r), l_max=int(lm),
                              m_max=int(mm))
             for p, n, r, lm, mm in zip(g["positions"], g["n_particle"], g["radii"], g["l_max"], g["m_max"])]
    ls = layers.LayerSystem([float(x) for x in g["thicknesses"]], [complex(x) for x in g["layer_n"]])
    offs = np.concatenate([[0], np.cumsum([flds.blocksize(p.l_max, p.m_max) for p in parts])])
    b = g["b_linear_w0"]
    for i, p in enumerate(parts):
        p.scattered_field = SphericalWaveExpansion(k=1, l_max=p.l_max, m_max=p.m_max, kind='outgoing',
                                                   reference_point=p.position)
        p.scattered_field.coefficients = b[offs[i]:offs[i + 1]]
    return parts, ls


def test_product_scattered_field_pwe_matches_reference():
    """The product's expansion of the reference solution (host particle sum), evaluated by the oracle,
    reproduces the reference's near field; validity bounds follow the reference's sums."""
    from smuthi_gb300.postprocessing import scattered_field as sf
    g = gc.load("vol5")
    parts, ls = _vol5_particles(g)
    pu, pd = sf.scattered_field_pwe(float(g["wavelength"]), parts, ls, ls.number_of_layers() - 1,
                                    k_parallel=g["nf_kpar"], azimuthal_angles=g["nf_azimuthal_angles"])
    zs = g["positions"][:, 2]
    assert (pu.lower_z, pu.upper_z) == (zs.max(), np.inf)
    assert (pd.lower_z, pd.upper_z) == (ls.lower_zlimit(1), zs.min())
    pts = g["nf_points"]
    for nm, pwe in (("up", pu), ("down", pd)):
        o = onf.PlaneWaveExpansion(pwe.k, pwe.k_parallel, pwe.azimuthal_angles, pwe.kind, pwe.reference_point,
                                   pwe.lower_z, pwe.upper_z)
        o.coefficients = pwe.coefficients
        E = np.array(o.field(pts[:, 0], pts[:, 1], pts[:, 2], 'E'))
        ref = g["nf_E_" + nm]
        if np.abs(ref).max() == 0:
            assert np.abs(E).max() == 0
        else:
            assert gc.relerr(E, ref) < 1e-12


def test_discrete_expansion_host_formula():
    """A single-wavenumber expansion is evaluated on the host with the reference's formula."""
    from smuthi_gb300.fields.expansions import PlaneWaveExpansion
    rng = np.random.default_rng(2)
    k = 0.015 + 0.0002j
    for kind in ("upgoing", "downgoing"):
        p = PlaneWaveExpansion(k, [0.008 + 0.0001j], [0.7], kind=kind, reference_point=[5, -3, 20], lower_z=0)
        p.coefficients = rng.standard_normal((2, 1, 1)) + 1j * rng.standard_normal((2, 1, 1))
        o = onf.PlaneWaveExpansion(k, [0.008 + 0.0001j], [0.7], kind, [5, -3, 20], 0)
        o.coefficients = p.coefficients
        x, y, z = rng.uniform(-100, 100, 7), rng.uniform(-100, 100, 7), rng.uniform(-50, 150, 7)
        for got, want in ((p.electric_field(x, y, z), o.field(x, y, z, 'E')),
                          (p.magnetic_field(x, y, z, 550.0), o.field(x, y, z, 'H', 550.0))):
            assert gc.relerr(np.array(got), np.array(want)) < 1e-14


def test_pwe_algebra():
    from smuthi_gb300.fields.expansions import PlaneWaveExpansion
    a = PlaneWaveExpansion(1.0, [0.1, 0.2], [0.0, 1.0], kind='upgoing', reference_point=[0, 0, 0], lower_z=0,
                           upper_z=10)
    b = PlaneWaveExpansion(1.0, [0.1, 0.2], [0.0, 1.0], kind='upgoing', reference_point=[0, 0, 0], lower_z=2,
                           upper_z=5)
    a.coefficients[:] = 1
    b.coefficients[:] = 2j
    s = a + b
    assert (s.lower_z, s.upper_z) == (2, 5) and np.all(s.coefficients == 1 + 2j)
    c = PlaneWaveExpansion(1.0, [0.1, 0.2], [0.0, 1.0], kind='downgoing', reference_point=[0, 0, 0])
    try:
        a + c
        raise AssertionError("incompatible expansions were added")
    except ValueError:
        pass
    # moving the reference point and back is the identity
    a.set_reference_point([3.0, -1.0, 2.0])
    a.set_reference_point([0, 0, 0])
    assert np.allclose(a.coefficients, 1)


def test_reference_point_translation_keeps_the_field():
    """Moving an expansion's reference point rephases its coefficients so that the field at every point
    is unchanged (the property of the reference's test_pwe_translation.py, here exact up to rounding
    because the quadrature nodes do not change)."""
    from smuthi_gb300.fields.expansions import PlaneWaveExpansion
    g = gc.load("pwe1")
    pts = g["points"]
    for kind in ("upgoing", "downgoing"):
        lo, hi = g["bounds_" + kind]
        p = PlaneWaveExpansion(complex(g["k"]), g["kpar"], g["alpha"], kind=kind,
                               reference_point=list(g["ref_" + kind]), lower_z=lo, upper_z=hi)
        p.coefficients = g["g_" + kind].copy()
        p.set_reference_point([300.0, 260.0, 100.0])
        o = onf.PlaneWaveExpansion(p.k, p.k_parallel, p.azimuthal_angles, kind, p.reference_point, lo, hi)
        o.coefficients = p.coefficients
        E = np.array(o.field(pts[:, 0], pts[:, 1], pts[:, 2], 'E'))
        assert gc.relerr(E, g["E_" + kind]) < 1e-9
