"""GPU parity of the volume-lookup path (particles at different heights in one layer).

Every call goes through the C ABI (``sg_set_volume_lookup`` and the operator / solver entry points).
References: the fixture ``vol5`` (the reference's own CPU volume lookup, run in the build container)
and the oracle (``oracle/volume.py``) on the product's tables, which are bit-equal to the
reference's. Tolerances: FP64 operator 1e-12 (relative 2-norm); FP64 solution and cross sections
1e-10 (both solvers driven to 1e-13); FP32 operator inside FP64 refinement: solution 1e-8.
"""
import numpy as np
import pytest

import golden_cases as gc
import oracle.volume as ovol

pytestmark = pytest.mark.gpu


def _spheres(g):
    from smuthi_gb300 import layers, particles
    parts = [particles.Sphere(position=list(p), refractive_index=complex(n), radius=float(r), l_max=int(lm),
                              m_max=int(mm))
             for p, n, r, lm, mm in zip(g["positions"], g["n_particle"], g["radii"], g["l_max"], g["m_max"])]
    ls = layers.LayerSystem([float(x) for x in g["thicknesses"]], [complex(x) for x in g["layer_n"]])
    return parts, ls, float(g["wavelength"])


def _system(parts, ls, wl, kp, resolution, kind, ctx):
    from smuthi_gb300.linearsystem import linear_system as lsm
    W = lsm.CouplingMatrixVolumeLookupCUDA(wl, parts, ls, k_parallel=kp, resolution=resolution,
                                           interpolator_kind=kind, context=ctx)
    for p in parts:
        p.t_matrix = p.compute_t_matrix(wl, ls.refractive_indices[ls.layer_number(p.position[2])])
    M = lsm.MasterMatrix(lsm.TMatrix(parts), W)
    return W, M


def _oracle(parts, W, kind):
    return ovol.VolumeLookupCPU(parts, W.lookup_table_plus, W.lookup_table_minus, W.rho_array, W.sum_z_array,
                                W.diff_z_array, kind)


def test_volume_matvec_fp64_matches_reference(gpu_context):
    g = gc.load("vol5")
    for kind in ("linear", "cubic"):
        parts, ls, wl = _spheres(g)
        W, M = _system(parts, ls, wl, g["kpar"], float(g["resolution"]), kind, gpu_context)
        x = g["x_" + kind]
        assert gc.relerr(W.linear_operator.matvec(x), g["Wx_" + kind]) < 1e-12
        assert gc.relerr(M.linear_operator.matvec(x), g["Mx_" + kind]) < 1e-12


def test_volume_hermite_matches_oracle(gpu_context):
    g = gc.load("vol5")
    parts, ls, wl = _spheres(g)
    W, _ = _system(parts, ls, wl, g["kpar"], float(g["resolution"]), "cubic_hermite", gpu_context)
    x = g["x_cubic"]
    assert gc.relerr(W.linear_operator.matvec(x), _oracle(parts, W, "cubic_hermite").matvec(x)) < 1e-12


def test_volume_solution_and_cross_sections(gpu_context):
    from smuthi_gb300 import fields as flds
    from smuthi_gb300 import initial_field as init
    from smuthi_gb300.postprocessing import far_field as ff
    g = gc.load("vol5")
    for tag in ("linear_w0", "linear_w1", "cubic_w0"):
        parts, ls, wl = _spheres(g)
        _system(parts, ls, wl, g["kpar"], float(g["resolution"]), tag.split("_w")[0], gpu_context)
        rhs = g["rhs_" + tag]
        b, info = gpu_context.gmres(rhs, rhs, 1e-13, restart=20, precision=0)
        assert info.converged == 1
        assert gc.relerr(b, g["b_" + tag]) < 1e-10
        offs = np.concatenate([[0], np.cumsum([flds.blocksize(p.l_max, p.m_max) for p in parts])])
        coefs = [b[offs[i]:offs[i + 1]] for i in range(len(parts))]
        pw = gc.plane_wave(g, int(tag.split("_w")[1]), init.PlaneWave)
        # particle sums on the GPU with per-particle height factors
        ext = ff.extinction_cross_section(initial_field=pw, particle_list=parts, layer_system=ls, coefficients=coefs,
                                          context=gpu_context)
        sca = ff.total_scattering_cross_section(initial_field=pw, particle_list=parts, layer_system=ls,
                                                coefficients=coefs, context=gpu_context)
        assert abs(ext - g["sigma_ext_" + tag]) <= 1e-10 * abs(g["sigma_ext_" + tag])
        assert abs(sca - g["sigma_sca_" + tag]) <= 1e-10 * abs(g["sigma_sca_" + tag])


def test_volume_mixed_precision_solve(gpu_context):
    from smuthi_gb300 import _lib
    g = gc.load("vol5")
    parts, ls, wl = _spheres(g)
    _system(parts, ls, wl, g["kpar"], float(g["resolution"]), "linear", gpu_context)
    for flags in (_lib.SG_FP32, _lib.SG_FP32 | _lib.SG_BLOCK_GMRES):
        rhs = np.stack([g["rhs_linear_w0"], g["rhs_linear_w1"]], axis=1)
        b, info = gpu_context.gmres(rhs, rhs, 1e-11, restart=20, precision=flags)
        assert info.converged == 2
        assert gc.relerr(b[:, 0], g["b_linear_w0"]) < 1e-8
        assert gc.relerr(b[:, 1], g["b_linear_w1"]) < 1e-8
        assert max(gpu_context.true_residual(rhs, b)) < 1e-10


def _random_volume_spheres(n, l_max, seed, box=1500.0, dmin=150.0):
    from smuthi_gb300 import particles
    rng = np.random.default_rng(seed)
    pts = []
    while len(pts) < n:
        p = np.array([rng.uniform(0, box), rng.uniform(0, box), rng.uniform(80.0, 180.0)])
        if all(np.hypot(*(p[:2] - q[:2])) > dmin for q in pts):
            pts.append(p)
    return [particles.Sphere(position=list(p), refractive_index=2.0 + 0.02j, radius=60.0, l_max=l_max, m_max=l_max)
            for p in pts]


@pytest.mark.parametrize("n, l_max, kinds, widths", [
    (40, 2, ("linear", "cubic"), (3, 12)),      # emitter split, RHS tiles of 8 with a partial tile
    (6, 4, ("linear", "cubic_hermite"), (1, 5)),  # blocksize 48: three rows per lane, RHS tiles of 4
])
def test_volume_multi_rhs_against_oracle(n, l_max, kinds, widths, gpu_context):
    from smuthi_gb300 import _lib
    from smuthi_gb300 import fields as flds
    from smuthi_gb300 import layers
    ls = layers.LayerSystem([0, 0], [1.52, 1])
    wl = 550.0
    kp = flds.reasonable_Sommerfeld_kpar_contour(wl, layer_refractive_indices=ls.refractive_indices)
    rng = np.random.default_rng(3)
    for kind in kinds:
        parts = _random_volume_spheres(n, l_max, seed=n)
        W, _ = _system(parts, ls, wl, kp, 10.0, kind, gpu_context)
        ref = _oracle(parts, W, kind)
        for R in widths:
            X = rng.standard_normal((W.shape[0], R)) + 1j * rng.standard_normal((W.shape[0], R))
            Y = gpu_context.coupling_matvec(X if R > 1 else X[:, 0], _lib.SG_FP64).reshape(W.shape[0], R)
            Yo = np.stack([ref.matvec(X[:, r]) for r in range(R)], axis=1)
            assert gc.relerr(Y, Yo) < 1e-12
            Y32 = gpu_context.coupling_matvec(X if R > 1 else X[:, 0], _lib.SG_FP32).reshape(W.shape[0], R)
            assert gc.relerr(Y32, Yo) < 1e-5


def test_volume_rejects_unsupported_modes(gpu_context):
    from smuthi_gb300 import _lib
    g = gc.load("vol5")
    parts, ls, wl = _spheres(g)
    W, _ = _system(parts, ls, wl, g["kpar"], float(g["resolution"]), "linear", gpu_context)
    x = g["x_linear"]
    for prec in (_lib.SG_DF64, _lib.SG_TF32X3):
        with pytest.raises(_lib.SmuthiGB300Error) as e:
            gpu_context.coupling_matvec(x, prec)
        assert e.value.code == 1
    rhs = g["rhs_linear_w0"]
    for flags in (_lib.SG_FP32 | _lib.SG_DF64, _lib.SG_FP32 | _lib.SG_PRECOND):
        with pytest.raises(_lib.SmuthiGB300Error) as e:
            gpu_context.gmres(rhs, rhs, 1e-8, precision=flags)
        assert e.value.code == 1
    # the context still works afterwards
    assert gc.relerr(W.linear_operator.matvec(x), g["Wx_linear"]) < 1e-12


def test_volume_simulation_api(gpu_context):
    """The reference-shaped Simulation takes the volume lookup for particles at different heights."""
    from smuthi_gb300 import initial_field as init, simulation
    from smuthi_gb300.linearsystem import linear_system as lsm
    from smuthi_gb300.postprocessing import far_field as ff
    g = gc.load("vol5")
    parts, ls, wl = _spheres(g)
    pw = gc.plane_wave(g, 0, init.PlaneWave)
    sim = simulation.Simulation(layer_system=ls, particle_list=parts, initial_field=pw, solver_type='gmres',
                                solver_tolerance=1e-13, store_coupling_matrix=False,
                                coupling_matrix_lookup_resolution=float(g["resolution"]),
                                coupling_matrix_interpolator_kind='linear', log_to_terminal=False)
    sim.run()
    assert isinstance(sim.linear_system.coupling_matrix, lsm.CouplingMatrixVolumeLookupCUDA)
    b = np.concatenate([p.scattered_field.coefficients for p in parts])
    assert gc.relerr(b, g["b_linear_w0"]) < 1e-10
    assert abs(ff.extinction_cross_section(sim) - g["sigma_ext_linear_w0"]) <= 1e-9 * g["sigma_ext_linear_w0"]
    assert abs(ff.total_scattering_cross_section(sim) - g["sigma_sca_linear_w0"]) <= 1e-9 * g["sigma_sca_linear_w0"]
