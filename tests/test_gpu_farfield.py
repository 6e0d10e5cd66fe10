"""GPU particle sum of the scattered plane-wave expansion against the host, and cross sections
against the reference's values.

``sg_farfield_sum`` evaluates, in FP64, the particle sum that dominates the far field; the angular
factors and the layer response stay on the host. Tolerances: the expansion within 1e-12 of the host
(relative 2-norm), extinction and total scattering cross sections of the reference's own solutions
within 1e-10 of the reference's cross sections.
"""
import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu


def _setup(name):
    from smuthi_gb300 import layers, particles
    g = gc.load(name)
    parts = [particles.Sphere(position=list(p), refractive_index=complex(n), radius=float(r), l_max=int(lm),
                              m_max=int(mm))
             for p, n, r, lm, mm in zip(g["positions"], g["n_particle"], g["radii"], g["l_max"], g["m_max"])]
    ln = [complex(x) if complex(x).imag else float(complex(x).real) for x in g["layer_n"]]
    ls = layers.LayerSystem([float(x) for x in g["thicknesses"]], ln)
    return g, parts, ls


@pytest.mark.parametrize("name", ["c5s", "c2s", "c3s"])
def test_scattered_pwe_gpu_matches_host(gpu_context, name):
    from smuthi_gb300.postprocessing import far_field as ff
    g, parts, ls = _setup(name)
    xy = np.array([p.position[:2] for p in parts])
    z = parts[0].position[2]
    lm, mm = parts[0].l_max, parts[0].m_max
    bs = 2 * lm * (lm + 2) if lm == mm else None
    rng = np.random.default_rng(3)
    coefs = rng.standard_normal((3, len(parts), bs)) + 1j * rng.standard_normal((3, len(parts), bs))
    wl = float(g["wavelength"])
    k_top = 2 * np.pi / wl * float(np.real(ls.refractive_indices[-1]))
    kp = np.linspace(0.0, 0.95 * k_top, 23)
    al = np.linspace(0.0, 2 * np.pi, 41)
    for layer in (0, ls.number_of_layers() - 1):
        host = ff.scattered_pwe(wl, ls, xy, z, lm, mm, coefs, layer, kp, al)
        dev = ff.scattered_pwe(wl, ls, xy, z, lm, mm, coefs, layer, kp, al, context=gpu_context)
        for h, d in zip(host, dev):
            assert gc.relerr(d, h) < 1e-12


@pytest.mark.parametrize("name", ["wg3", "c5s", "c3s"])
def test_cross_sections_of_reference_solutions(gpu_context, name):
    from smuthi_gb300 import initial_field as init
    from smuthi_gb300.postprocessing import far_field as ff
    g, parts, ls = _setup(name)
    if len({(p.l_max, p.m_max) for p in parts}) != 1:
        pytest.skip("cross sections are provided for one multipole cut-off")
    for key in [k for k in g if k.startswith("b_")]:
        tag = key[2:]
        pw = gc.plane_wave(g, int(tag.split("_w")[1]), init.PlaneWave)
        coef = g[key].reshape(len(parts), -1)
        ext = ff.extinction_cross_section(initial_field=pw, particle_list=parts, layer_system=ls, coefficients=coef,
                                          context=gpu_context)
        sca = ff.total_scattering_cross_section(initial_field=pw, particle_list=parts, layer_system=ls,
                                                coefficients=coef, context=gpu_context)
        assert abs(ext - g["sigma_ext_" + tag]) <= 1e-10 * abs(g["sigma_ext_" + tag])
        assert abs(sca - g["sigma_sca_" + tag]) <= 1e-10 * abs(g["sigma_sca_" + tag])


def test_farfield_argument_checks(gpu_context):
    from smuthi_gb300 import _lib
    with pytest.raises(_lib.SmuthiGB300Error):  # m_of_n outside [-m_max, m_max]: rejected before any launch
        gpu_context.farfield_sum_dev(1, 8, 2, 1, 8, 0, [0, 1], 1, 8, 8, 1, 8, 8)
    with pytest.raises(_lib.SmuthiGB300Error):  # empty angular grid
        gpu_context.farfield_sum_dev(1, 8, 1, 1, 8, 0, [0], 1, 8, 8, 0, 8, 8)
