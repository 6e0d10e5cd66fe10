"""Initial-field coefficients of a batch of plane waves on the GPU (``sg_plane_wave_swe``) against the
reference's own values in the golden fixtures and against the host restatement."""
import numpy as np
import pytest

import golden_cases as gc
from test_initial_field_host import _layers, _waves

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", gc.available())
def test_batched_plane_wave_swe_matches_reference(name, gpu_context):
    from smuthi_gb300 import initial_field as init
    g = gc.load(name)
    ls = _layers(g)
    kind = [k for k in g if k.startswith("a_")][0].split("_")[1]
    qs = _waves(g)
    waves = [gc.plane_wave(g, q, init.PlaneWave) for q in qs]
    pos = np.asarray(g["positions"], float)
    lms = list(zip(g["l_max"], g["m_max"]))
    out = [[None] * len(pos) for _ in qs]
    for key in sorted(set(lms)):
        idx = [i for i, lm in enumerate(lms) if lm == key]
        a = init.swe_coefficients_batch(waves, pos[idx], ls, int(key[0]), int(key[1]), gpu_context)
        assert a.shape == (len(qs), len(idx), a.shape[2])
        for w in range(len(qs)):
            for r, i in enumerate(idx):
                out[w][i] = a[w, r]
    for w, q in enumerate(qs):
        assert gc.relerr(np.concatenate(out[w]), g["a_%s_w%d" % (kind, q)]) < 1e-12, (name, q)


def test_batched_plane_wave_swe_film_many_waves(gpu_context):
    """Sixteen waves from both half-spaces, both polarisations, in a three-layer film (two plane-wave
    components per wave in the film): GPU against the host restatement."""
    from smuthi_gb300 import initial_field as init, layers
    ls = layers.LayerSystem([0, 300, 0], [1.52, 1.8 + 0.01j, 1.0])
    rng = np.random.default_rng(5)
    pos = np.column_stack([rng.uniform(-3000, 3000, (500, 2)), np.full(500, 150.0)])
    waves = [init.PlaneWave(550.0, polar_angle=(rng.uniform(0, 0.8) if q % 2 else np.pi - rng.uniform(0, 0.8)),
                            azimuthal_angle=rng.uniform(0, 2 * np.pi), polarization=q % 2,
                            reference_point=[10.0, -20.0, 5.0]) for q in range(16)]
    a = init.swe_coefficients_batch(waves, pos, ls, 3, 3, gpu_context)
    host = np.stack([w.swe_coefficients(pos, ls, 3, 3) for w in waves])
    assert gc.relerr(a, host) < 1e-13
