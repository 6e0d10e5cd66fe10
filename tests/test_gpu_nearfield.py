"""GPU near-field evaluation (``sg_pwe_field``) against the reference's own fields and the oracle.

Tolerance: relative 2-norm 1e-12 (FP64 on both sides, same quadrature).
"""
import numpy as np
import pytest

import golden_cases as gc
import oracle.nearfield as onf

pytestmark = pytest.mark.gpu


def test_pwe_fields_match_reference(gpu_context):
    from smuthi_gb300.fields.expansions import PlaneWaveExpansion
    g = gc.load("pwe1")
    pts = g["points"]
    for kind in ("upgoing", "downgoing"):
        lo, hi = g["bounds_" + kind]
        p = PlaneWaveExpansion(complex(g["k"]), g["kpar"], g["alpha"], kind=kind, reference_point=list(g["ref_" + kind]),
                               lower_z=lo, upper_z=hi)
        p.coefficients = g["g_" + kind]
        E = np.array(p.electric_field(pts[:, 0], pts[:, 1], pts[:, 2], context=gpu_context))
        H = np.array(p.magnetic_field(pts[:, 0], pts[:, 1], pts[:, 2], float(g["wavelength"]), context=gpu_context))
        assert gc.relerr(E, g["E_" + kind]) < 1e-12
        assert gc.relerr(H, g["H_" + kind]) < 1e-12


def test_scattered_near_field_matches_reference(gpu_context):
    from smuthi_gb300.postprocessing import scattered_field as sf
    from test_nearfield_host import _vol5_particles
    g = gc.load("vol5")
    parts, ls = _vol5_particles(g)
    pu, pd = sf.scattered_field_pwe(float(g["wavelength"]), parts, ls, ls.number_of_layers() - 1,
                                    k_parallel=g["nf_kpar"], azimuthal_angles=g["nf_azimuthal_angles"],
                                    context=gpu_context)
    pts = g["nf_points"]
    E = np.array(pu.electric_field(pts[:, 0], pts[:, 1], pts[:, 2], context=gpu_context))
    assert gc.relerr(E, g["nf_E_up"]) < 1e-11
    assert np.abs(np.array(pd.electric_field(pts[:, 0], pts[:, 1], pts[:, 2], context=gpu_context))).max() == 0


def test_many_points_against_oracle(gpu_context):
    """2000 points (several point blocks and kappa splits), odd grid sizes, a real and a complex contour."""
    from smuthi_gb300 import fields as flds
    from smuthi_gb300.fields.expansions import PlaneWaveExpansion
    rng = np.random.default_rng(9)
    k = flds.angular_frequency(600.0) * 1.45
    for kp in (np.linspace(0, 1.2 * k.real, 61),
               flds.reasonable_Sommerfeld_kpar_contour(600.0, layer_refractive_indices=[1.45, 1.0],
                                                       neff_resolution=5e-2)):
        al = np.sort(rng.uniform(0, 2 * np.pi, 23))
        p = PlaneWaveExpansion(k, kp, al, kind='upgoing', reference_point=[0, 0, 0], lower_z=0)
        p.coefficients = rng.standard_normal(p.coefficients.shape) + 1j * rng.standard_normal(p.coefficients.shape)
        o = onf.PlaneWaveExpansion(k, kp, al, 'upgoing', [0, 0, 0], 0)
        o.coefficients = p.coefficients
        n = 2000
        x, y, z = rng.uniform(-500, 500, n), rng.uniform(-500, 500, n), rng.uniform(-20, 300, n)
        E = np.array(p.electric_field(x, y, z, context=gpu_context))
        assert gc.relerr(E, np.array(o.field(x, y, z, 'E'))) < 1e-12
        H = np.array(p.magnetic_field(x, y, z, 600.0, context=gpu_context))
        assert gc.relerr(H, np.array(o.field(x, y, z, 'H', 600.0))) < 1e-12


def test_pwe_field_argument_errors(gpu_context):
    from smuthi_gb300 import _lib
    import torch
    dev = torch.device("cuda", gpu_context.device)
    buf = torch.zeros(64, dtype=torch.complex128, device=dev)
    p = buf.data_ptr()
    with pytest.raises(_lib.SmuthiGB300Error) as e:  # a single kappa node is the host's discrete case
        gpu_context.pwe_field_dev(0, 4, p, p, p, 1, p, p, 4, p, p, 1.0, 1.0, p)
    assert e.value.code == 1
    with pytest.raises(_lib.SmuthiGB300Error) as e:
        gpu_context.pwe_field_dev(2, 4, p, p, p, 4, p, p, 4, p, p, 1.0, 1.0, p)
    assert e.value.code == 1
