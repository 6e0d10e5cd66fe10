"""LinearSystem picks the coupling matrix the reference would (linear_system.py:149-252). No GPU:
the GPU classes are replaced by recording stand-ins."""
import numpy as np
import pytest


def _system(z_values, kind='linear'):
    from smuthi_gb300 import initial_field as init
    from smuthi_gb300 import layers, particles
    from smuthi_gb300.linearsystem import linear_system as lsm
    parts = [particles.Sphere(position=[300.0 * i, 0.0, z], refractive_index=2.0, radius=80.0, l_max=2, m_max=2)
             for i, z in enumerate(z_values)]
    ls = layers.LayerSystem([0, 0], [1.52, 1])
    pw = init.PlaneWave(vacuum_wavelength=550.0, polar_angle=np.pi, azimuthal_angle=0.0, polarization=0)
    return lsm.LinearSystem(parts, pw, ls, solver_type='gmres', store_coupling_matrix=False,
                            coupling_matrix_lookup_resolution=5.0, interpolator_kind=kind)


@pytest.fixture
def recorded(monkeypatch):
    from smuthi_gb300.linearsystem import linear_system as lsm
    from smuthi_gb300.utility import cuda as cu
    calls = []

    def fake(name):
        def ctor(**kw):
            calls.append((name, kw))
            return name
        return ctor

    monkeypatch.setattr(lsm, "CouplingMatrixRadialLookupCUDA", fake("radial"))
    monkeypatch.setattr(lsm, "CouplingMatrixVolumeLookupCUDA", fake("volume"))
    monkeypatch.setattr(cu, "use_gpu", True)
    return calls


def test_same_height_takes_radial_lookup(recorded):
    ls = _system([100.0, 100.0, 100.0])
    ls.compute_coupling_matrix()
    assert ls.coupling_matrix == "radial" and recorded[0][1]["interpolator_kind"] == "linear"


def test_different_heights_take_volume_lookup(recorded):
    ls = _system([100.0, 130.0, 90.0], kind='cubic')
    ls.compute_coupling_matrix()
    assert ls.coupling_matrix == "volume"
    assert recorded[0][1]["interpolator_kind"] == "cubic" and recorded[0][1]["resolution"] == 5.0


def test_unknown_kind_warns_and_uses_linear(recorded):
    ls = _system([100.0, 130.0], kind='quintic')
    with pytest.warns(UserWarning):
        ls.compute_coupling_matrix()
    assert recorded[0][1]["interpolator_kind"] == "linear"


def test_unsupported_branches_raise(recorded):
    from smuthi_gb300 import layers
    ls = _system([100.0, 100.0])
    ls.solver_type = 'LU'
    with pytest.raises(NotImplementedError):
        ls.compute_coupling_matrix()
    ls = _system([100.0, 100.0])
    ls.layer_system = layers.LayerSystem([0, 150, 0], [1.52, 1.3, 1])
    with pytest.raises(NotImplementedError):  # particles in two layers (z = 100 in layer 1, 400 in layer 2)
        ls.particle_list[1].position[2] = 400.0
        ls.compute_coupling_matrix()
