"""Initial-field coefficients of plane waves at the particles (host restatement) against the
reference's own values in the golden fixtures (`a_<kind>_w<q>`: the regular SWE coefficients of wave q
at every particle, smuthi/initial_field.py:284-329 through smuthi/fields/transformations.py:77-131)."""
import numpy as np
import pytest

import golden_cases as gc


def _layers(g):
    from smuthi_gb300 import layers
    ln = [complex(x) if complex(x).imag else float(complex(x).real) for x in g["layer_n"]]
    return layers.LayerSystem([float(x) for x in g["thicknesses"]], ln)


def _waves(g):
    return sorted({int(k.rsplit("_w", 1)[1]) for k in g if k.startswith("a_")})


@pytest.mark.parametrize("name", gc.available())
def test_swe_coefficients_match_reference(name):
    from smuthi_gb300 import initial_field as init
    g = gc.load(name)
    ls = _layers(g)
    kind = [k for k in g if k.startswith("a_")][0].split("_")[1]
    for q in _waves(g):
        pw = gc.plane_wave(g, q, init.PlaneWave)
        blocks = [pw.swe_coefficients([p], ls, int(lm), int(mm))[0]
                  for p, lm, mm in zip(g["positions"], g["l_max"], g["m_max"])]
        assert gc.relerr(np.concatenate(blocks), g["a_%s_w%d" % (kind, q)]) < 1e-12, (name, q)


def test_component_terms_rebuild_host_coefficients():
    """Each plane-wave component's (wavevector, per-index factors) rebuild the host coefficients: the
    split the GPU kernel sg_plane_wave_swe evaluates."""
    from smuthi_gb300 import initial_field as init
    g = gc.load("c5s")
    ls = _layers(g)
    pos = np.asarray(g["positions"], float)
    for q in _waves(g):
        pw = gc.plane_wave(g, q, init.PlaneWave)
        layer = ls.layer_number(pos[0, 2])
        acc = np.zeros((len(pos), 30), complex)
        for pwe in pw.plane_wave_expansion(ls, layer):
            kr, amp = init.component_terms(pwe, 3, 3)
            d = pos - kr[4:7]
            acc += np.exp(1j * (kr[0] * d[:, [0]] + kr[1] * d[:, [1]] + complex(kr[2], kr[3]) * d[:, [2]])) * amp
        assert gc.relerr(acc.ravel(), g["a_linear_w%d" % q]) < 1e-12
