"""GPU parity of the sm_103a path against the reference's own outputs and the oracle.

Every call goes through the C ABI (``include/smuthi_gb300.h``) via ctypes.
Tolerances: FP64 operator vs reference 1e-12 (relative 2-norm); plain FP64
solution and cross sections vs reference 1e-10 (both solvers driven to a
relative residual of 1e-13); mixed precision: FP64-true residual 1e-6 and
cross sections within 1e-6 of the reference.
"""
import numpy as np
import pytest

import golden_cases as gc
import oracle.physics as ophys
import oracle.solve as osv

pytestmark = pytest.mark.gpu

CASES = gc.available()


def _product_system(g, kind, ctx):
    from smuthi_gb300 import layers, particles
    from smuthi_gb300.linearsystem import linear_system as lsm
    parts = [particles.Sphere(position=list(p), refractive_index=complex(n), radius=float(r), l_max=int(lm),
                              m_max=int(mm))
             for p, n, r, lm, mm in zip(g["positions"], g["n_particle"], g["radii"], g["l_max"], g["m_max"])]
    ln = [complex(x) if complex(x).imag else float(complex(x).real) for x in g["layer_n"]]
    ls = layers.LayerSystem([float(x) for x in g["thicknesses"]], ln)
    wl = float(g["wavelength"])
    W = lsm.CouplingMatrixRadialLookupCUDA(wl, parts, ls, k_parallel=g["kpar"], resolution=float(g["resolution"]),
                                           interpolator_kind=kind, context=ctx)
    for p in parts:
        p.t_matrix = p.compute_t_matrix(wl, ls.refractive_indices[ls.layer_number(p.position[2])])
    T = lsm.TMatrix(parts)
    M = lsm.MasterMatrix(T, W)
    return parts, ls, wl, W, M


def _kinds(g):
    return [k for k in ("linear", "cubic") if "x_" + k in g]


@pytest.mark.parametrize("name", CASES)
def test_coupling_and_master_matvec_fp64(name, gpu_context):
    g = gc.load(name)
    for kind in _kinds(g):
        parts, ls, wl, W, M = _product_system(g, kind, gpu_context)
        x = g["x_" + kind]
        assert gc.relerr(W.linear_operator.matvec(x), g["Wx_" + kind]) < 1e-12
        assert gc.relerr(M.linear_operator.matvec(x), g["Mx_" + kind]) < 1e-12


@pytest.mark.parametrize("name", CASES)
def test_plain_fp64_solution_and_cross_sections(name, gpu_context):
    from smuthi_gb300.postprocessing import far_field as ff
    from smuthi_gb300 import initial_field as init
    g = gc.load(name)
    for key in [k for k in g if k.startswith("b_")]:
        tag = key[2:]
        kind = tag.split("_w")[0]
        parts, ls, wl, W, M = _product_system(g, kind, gpu_context)
        rhs = g["rhs_" + tag]
        b, info = gpu_context.gmres(rhs, rhs, 1e-13, restart=20, precision=0)
        assert info.converged == 1
        assert gc.relerr(b, g[key]) < 1e-10
        if len({(p.l_max, p.m_max) for p in parts}) == 1:
            pw = gc.plane_wave(g, int(tag.split("_w")[1]), init.PlaneWave)
            coef = b.reshape(len(parts), -1)
            ext = ff.extinction_cross_section(initial_field=pw, particle_list=parts, layer_system=ls, coefficients=coef)
            assert abs(ext - g["sigma_ext_" + tag]) <= 1e-10 * abs(g["sigma_ext_" + tag])
            if name in ("wg3", "c5s", "c3s"):
                sca = ff.total_scattering_cross_section(initial_field=pw, particle_list=parts, layer_system=ls,
                                                        coefficients=coef)
                assert abs(sca - g["sigma_sca_" + tag]) <= 1e-10 * abs(g["sigma_sca_" + tag])


@pytest.mark.parametrize("name", ["c1", "c5s", "c3s"])
def test_mixed_precision_solution(name, gpu_context):
    from smuthi_gb300.postprocessing import far_field as ff
    from smuthi_gb300 import initial_field as init
    g = gc.load(name)
    key = [k for k in g if k.startswith("b_")][0]
    tag = key[2:]
    kind = tag.split("_w")[0]
    parts, ls, wl, W, M = _product_system(g, kind, gpu_context)
    rhs = g["rhs_" + tag]
    b, info = gpu_context.gmres(rhs, rhs, 1e-6, restart=20, precision=1)
    assert info.converged == 1
    assert info.max_rel_residual <= 1e-6
    # FP64-true residual, recomputed independently through the C ABI
    assert gpu_context.true_residual(rhs, b)[0] <= 1e-6
    assert info.fp64_matvecs <= 5
    pw = gc.plane_wave(g, int(tag.split("_w")[1]), init.PlaneWave)
    ext = ff.extinction_cross_section(initial_field=pw, particle_list=parts, layer_system=ls,
                                      coefficients=b.reshape(len(parts), -1))
    assert abs(ext - g["sigma_ext_" + tag]) <= 1e-6 * abs(g["sigma_ext_" + tag])


@pytest.mark.parametrize("name", ["wg3", "c1"])
def test_fp32_operator_close_to_fp64(name, gpu_context):
    g = gc.load(name)
    kind = _kinds(g)[0]
    parts, ls, wl, W, M = _product_system(g, kind, gpu_context)
    x = g["x_" + kind]
    y64 = gpu_context.coupling_matvec(x, 0)
    y32 = gpu_context.coupling_matvec(x, 1)
    assert gc.relerr(y32, y64) < 2e-5


def test_multi_rhs_linearity_and_lockstep(gpu_context):
    g = gc.load("c5s")
    parts, ls, wl, W, M = _product_system(g, "linear", gpu_context)
    x = g["x_linear"]
    X = np.stack([x, 2 * x, 1j * x, x.conj()], axis=1)
    Y = gpu_context.coupling_matvec(np.ascontiguousarray(X), 0)
    y = gpu_context.coupling_matvec(x, 0)
    yc = gpu_context.coupling_matvec(np.ascontiguousarray(x.conj()), 0)
    assert gc.relerr(Y[:, 0], y) < 1e-15
    assert gc.relerr(Y[:, 1], 2 * y) < 1e-14
    assert gc.relerr(Y[:, 2], 1j * y) < 1e-14
    assert gc.relerr(Y[:, 3], yc) < 1e-15
    rhs = np.stack([g["rhs_linear_w0"], g["rhs_linear_w1"]], axis=1)
    B, info = gpu_context.gmres(np.ascontiguousarray(rhs), np.ascontiguousarray(rhs), 1e-13, precision=0)
    assert info.converged == 2
    assert gc.relerr(B[:, 0], g["b_linear_w0"]) < 1e-10
    assert gc.relerr(B[:, 1], g["b_linear_w1"]) < 1e-10


def test_cubic_hermite_matches_oracle(gpu_context):
    g = gc.load("wg3")
    parts, ls, wl, W, M = _product_system(g, "cubic_hermite", gpu_context)
    oparts, _, _ = gc.oracle_inputs(g)
    Wo = osv.RadialLookupCPU(oparts, g["table"], g["rho_grid"], "cubic_hermite")
    x = g["x_linear"]
    assert gc.relerr(W.linear_operator.matvec(x), Wo.matvec(x)) < 1e-12


def test_determinism_fp64(gpu_context):
    g = gc.load("c1")
    parts, ls, wl, W, M = _product_system(g, "linear", gpu_context)
    x = g["x_linear"]
    a = gpu_context.master_matvec(x, 0)
    b = gpu_context.master_matvec(x, 0)
    assert np.array_equal(a, b)


def test_errors_are_reported(gpu_context):
    from smuthi_gb300 import _lib
    g = gc.load("wg3")
    _product_system(g, "linear", gpu_context)
    x = g["x_linear"].copy()
    x[3] = np.nan
    with pytest.raises(_lib.SmuthiGB300Error) as e:
        gpu_context.coupling_matvec(x, 0)
    assert e.value.code == _lib.SG_ERR_NAN
    with pytest.raises(_lib.SmuthiGB300Error) as e:
        gpu_context.set_lookup(7, g["table"], g["rho_grid"][0], 5.0)
    assert e.value.code == _lib.SG_ERR_ARG
    with pytest.raises(_lib.SmuthiGB300Error) as e:  # grid too short for the particle distances
        gpu_context.set_lookup("linear", g["table"][:10], g["rho_grid"][0], 5.0)
    assert e.value.code == _lib.SG_ERR_ARG
    with pytest.raises(_lib.SmuthiGB300Error):
        gpu_context.set_particles(np.zeros((2, 2)), [0, 0], [1, 1], 30, np.zeros(30))


def test_simulation_api_end_to_end(gpu_context):
    """The reference-shaped Simulation API on the GPU reproduces the reference solution."""
    import smuthi_gb300.fields as flds
    from smuthi_gb300 import initial_field as init, layers, particles, simulation
    g = gc.load("c5s")
    parts = [particles.Sphere(position=list(p), refractive_index=complex(n), radius=float(r), l_max=int(lm),
                              m_max=int(mm))
             for p, n, r, lm, mm in zip(g["positions"], g["n_particle"], g["radii"], g["l_max"], g["m_max"])]
    ls = layers.LayerSystem([float(x) for x in g["thicknesses"]], [float(complex(x).real) for x in g["layer_n"]])
    pw = gc.plane_wave(g, 0, init.PlaneWave)
    sim = simulation.Simulation(layer_system=ls, particle_list=parts, initial_field=pw, solver_type='gmres',
                                solver_tolerance=1e-13, store_coupling_matrix=False,
                                coupling_matrix_lookup_resolution=float(g["resolution"]),
                                coupling_matrix_interpolator_kind='linear', log_to_terminal=False)
    sim.run()
    np.testing.assert_array_equal(flds.default_Sommerfeld_k_parallel_array, g["kpar"])
    b = np.concatenate([p.scattered_field.coefficients for p in parts])
    assert gc.relerr(b, g["b_linear_w0"]) < 1e-10
    # cross sections through the simulation: the particle sums run on the simulation's GPU context
    from smuthi_gb300.postprocessing import far_field as ff
    assert abs(ff.extinction_cross_section(sim) - g["sigma_ext_linear_w0"]) <= 1e-9 * abs(g["sigma_ext_linear_w0"])
    assert abs(ff.total_scattering_cross_section(sim) - g["sigma_sca_linear_w0"]) <= 1e-9 * abs(
        g["sigma_sca_linear_w0"])


def test_full_size_c2_properties(gpu_context):
    """Full c2 shape (2000 spheres, cubic): oracle rows, FP32/FP64 agreement, linearity."""
    from smuthi_gb300 import workloads
    import smuthi_gb300.fields as flds
    spec = workloads.build("c2", seed=0)
    from smuthi_gb300 import layers, particles
    parts = [particles.Sphere(position=list(p), refractive_index=spec["n_particle"], radius=spec["radius"],
                              l_max=3, m_max=3) for p in spec["positions"]]
    ls = layers.LayerSystem(*spec["layers"])
    wl = spec["wavelength"]
    kp = flds.reasonable_Sommerfeld_kpar_contour(wl, layer_refractive_indices=ls.refractive_indices)
    from smuthi_gb300.linearsystem import linear_system as lsm
    W = lsm.CouplingMatrixRadialLookupCUDA(wl, parts, ls, k_parallel=kp, resolution=spec["resolution"],
                                           interpolator_kind="cubic", context=gpu_context)
    rng = np.random.default_rng(5)
    x = rng.standard_normal(W.shape[0]) + 1j * rng.standard_normal(W.shape[0])
    y = gpu_context.coupling_matvec(x, 0)
    oparts = [ophys.Sphere(p.position, p.refractive_index, p.radius, 3, 3) for p in parts]
    Wo = osv.RadialLookupCPU.__new__(osv.RadialLookupCPU)
    # restricted oracle: 6 receiving particles against all emitters
    rows = np.array([0, 17, 512, 999, 1500, 1999])
    Wo.__init__(oparts, W.lookup_table, W.radial_distance_array, "cubic")
    yo = Wo.matvec(x, rows=rows)
    sel = np.concatenate([np.arange(r * 30, r * 30 + 30) for r in rows])
    assert gc.relerr(y[sel], yo[sel]) < 1e-11
    y32 = gpu_context.coupling_matvec(x, 1)
    assert gc.relerr(y32, y) < 2e-5
    x2 = rng.standard_normal(W.shape[0]) + 0j
    y2 = gpu_context.coupling_matvec(x2, 0)
    y12 = gpu_context.coupling_matvec(x + 0.5j * x2, 0)
    assert gc.relerr(y12, y + 0.5j * y2) < 1e-13


@pytest.mark.parametrize("name", ["c5s", "c1"])
def test_block_gmres_mixed(name, gpu_context):
    """Block GMRES correction solves (one Krylov space for all RHS) reach the FP64-true tolerance."""
    from smuthi_gb300 import _lib
    g = gc.load(name)
    kind = _kinds(g)[0]
    parts, ls, wl, W, M = _product_system(g, kind, gpu_context)
    keys = sorted(k for k in g if k.startswith("rhs_"))
    rng = np.random.default_rng(2)
    cols = [g[k] for k in keys]
    while len(cols) < 3:  # extra right-hand sides: perturbed copies (not collinear)
        cols.append(cols[0] * (1 + 0.3 * rng.standard_normal(len(cols[0]))))
    B = np.ascontiguousarray(np.stack(cols, axis=1))
    X, info = gpu_context.gmres(B, np.zeros_like(B), 1e-6, restart=20, precision=_lib.SG_FP32 | _lib.SG_BLOCK_GMRES)
    assert info.converged == B.shape[1]
    assert gpu_context.true_residual(B, X).max() <= 1e-6
    for q, k in enumerate(keys):
        bk = "b_" + k[4:]
        if bk in g:
            assert gc.relerr(X[:, q], g[bk]) < 1e-4


@pytest.mark.parametrize("name", CASES)
def test_df64_operator_matches_fp64(name, gpu_context):
    """The double-float operator (two FP32 words per value on the FP32 pipe) is FP64-grade."""
    from smuthi_gb300 import _lib
    g = gc.load(name)
    for kind in _kinds(g):
        parts, ls, wl, W, M = _product_system(g, kind, gpu_context)
        x = g["x_" + kind]
        assert gc.relerr(gpu_context.coupling_matvec(x, _lib.SG_DF64), gpu_context.coupling_matvec(x, 0)) < 1e-12
        assert gc.relerr(gpu_context.coupling_matvec(x, _lib.SG_DF64), g["Wx_" + kind]) < 1e-12
        assert gc.relerr(gpu_context.master_matvec(x, _lib.SG_DF64), g["Mx_" + kind]) < 1e-12
        X = np.ascontiguousarray(np.stack([x, 1j * x, x.conj()], axis=1))  # RHS tiles of 1, 2, 4 columns
        Y = gpu_context.master_matvec(X, _lib.SG_DF64)
        assert gc.relerr(Y, gpu_context.master_matvec(X, 0)) < 1e-12


@pytest.mark.parametrize("name", ["c1", "c5s", "c3s"])
def test_mixed_solution_with_df64_residuals(name, gpu_context):
    """Refinement residuals in double-float still give an FP64-true residual below the tolerance."""
    from smuthi_gb300 import _lib
    g = gc.load(name)
    keys = sorted(k for k in g if k.startswith("b_"))
    kind = keys[0][2:].split("_w")[0]
    parts, ls, wl, W, M = _product_system(g, kind, gpu_context)
    B = np.ascontiguousarray(np.stack([g["rhs_" + k[2:]] for k in keys], axis=1))
    X, info = gpu_context.gmres(B, np.zeros_like(B), 1e-6, restart=20, precision=_lib.SG_FP32 | _lib.SG_DF64)
    assert info.converged == B.shape[1]
    assert gpu_context.true_residual(B, X).max() <= 1e-6
    for q, k in enumerate(keys):
        assert gc.relerr(X[:, q], g[k]) < 1e-4


@pytest.mark.parametrize("name", ["c5s", "c2s", "c1"])
def test_tensor_core_operator_matches_fp64(name, gpu_context):
    """The tcgen05 3xTF32 operator (accumulators drained every 8 emitters into an FP32 total) within
    5e-6 of the FP64 operator for 16, 32 and 64 right-hand sides, with the self pairs included."""
    from smuthi_gb300 import _lib
    g = gc.load(name)
    kind = _kinds(g)[0]
    parts, ls, wl, W, M = _product_system(g, kind, gpu_context)
    x = g["x_" + kind]
    rng = np.random.default_rng(4)
    for R in (16, 32, 64):
        X = np.ascontiguousarray(np.stack([x * np.exp(2j * np.pi * rng.random()) * (1 + 0.5 * rng.random())
                                           for _ in range(R)], axis=1))
        for fn in (gpu_context.coupling_matvec, gpu_context.master_matvec):
            ref = fn(X, _lib.SG_FP64)
            tc = fn(X, _lib.SG_TF32X3)
            assert gc.relerr(tc, ref) < 5e-6, (R, fn.__name__, gc.relerr(tc, ref))


@pytest.mark.parametrize("count", [1, 2, 3, 5])
def test_one_and_two_particle_systems(count, gpu_context):
    """Smallest systems (the self pair only, one pair, odd counts whose last receiver pair has one
    particle): every precision against the oracle's FP64 operator, both tensor-core operators on 16
    RHS, and the plain and chosen solves to their tolerances."""
    from smuthi_gb300 import _lib
    g = gc.load("c5s")
    sub = {k: g[k] for k in g}
    for key in ("positions", "n_particle", "radii", "l_max", "m_max"):
        sub[key] = g[key][:count]
    parts, ls, wl, W, M = _product_system(sub, "linear", gpu_context)
    oparts, _, _ = gc.oracle_inputs(sub)
    Wo = osv.RadialLookupCPU(oparts, W.lookup_table, W.radial_distance_array, "linear")
    rng = np.random.default_rng(count)
    x = rng.standard_normal(W.shape[0]) + 1j * rng.standard_normal(W.shape[0])
    ref = Wo.matvec(x)
    assert gc.relerr(W.linear_operator.matvec(x), ref) < 1e-12
    assert gc.relerr(gpu_context.coupling_matvec(x, _lib.SG_DF64), ref) < 1e-12
    assert gc.relerr(gpu_context.coupling_matvec(x, _lib.SG_FP32), ref) < 1e-5
    X = np.ascontiguousarray(np.stack([x * np.exp(0.3j * q) for q in range(16)], axis=1))
    Y = np.stack([Wo.matvec(X[:, q]) for q in range(16)], axis=1)
    assert gc.relerr(gpu_context.coupling_matvec(X, _lib.SG_TF32X3), Y) < 5e-6
    if count >= 2:
        gpu_context.fp32_set_kernel(16, 5, 16)
        assert gc.relerr(gpu_context.coupling_matvec(X, _lib.SG_FP32), Y) < 5e-6
    b = np.ascontiguousarray(x)
    for prec, tol in ((_lib.SG_FP64, 1e-12), (_lib.SG_FP32 | _lib.SG_DF64, 1e-6)):
        sol, info = gpu_context.gmres(b, np.zeros_like(b), tol, precision=prec)
        assert info.converged == 1
        assert gpu_context.true_residual(b, sol)[0] <= tol


def test_simulation_chosen_form_two_waves(gpu_context):
    """The chosen form through the reference-shaped API: two plane waves solved as one batch with the
    mixed-precision operator, double-float residuals and the learned preconditioner. At a relative
    residual of 1e-6 both cross sections of each wave are within 1e-6 of the reference's; solved to
    1e-10 both solutions are within 1e-6 of the reference's."""
    from smuthi_gb300 import initial_field as init, layers, particles, simulation
    from smuthi_gb300.postprocessing import far_field as ff
    g = gc.load("c5s")
    ls = layers.LayerSystem([float(x) for x in g["thicknesses"]], [float(complex(x).real) for x in g["layer_n"]])
    waves = [gc.plane_wave(g, q, init.PlaneWave) for q in range(2)]
    for tol in (1e-6, 1e-10):
        parts = [particles.Sphere(position=list(p), refractive_index=complex(n), radius=float(r), l_max=int(lm),
                                  m_max=int(mm))
                 for p, n, r, lm, mm in zip(g["positions"], g["n_particle"], g["radii"], g["l_max"], g["m_max"])]
        sim = simulation.Simulation(layer_system=ls, particle_list=parts, initial_field=waves, solver_type='gmres',
                                    solver_tolerance=tol, store_coupling_matrix=False,
                                    coupling_matrix_lookup_resolution=float(g["resolution"]),
                                    coupling_matrix_interpolator_kind='linear', log_to_terminal=False,
                                    precision='mixed', residual='df64', preconditioner='learned', restart=32)
        sim.run()
        info = sim.linear_system.solve_info
        assert info["converged"] == 2 and info["max_rel_residual"] <= tol
        assert sim.linear_system.preconditioner_name == "precond_c5"
        for q in range(2):
            sim.select_wave(q)
            b = np.concatenate([p.scattered_field.coefficients for p in parts])
            if tol == 1e-10:
                assert gc.relerr(b, g["b_linear_w%d" % q]) < 1e-6
            else:
                for fn, key in ((ff.extinction_cross_section, "sigma_ext"), (ff.total_scattering_cross_section,
                                                                              "sigma_sca")):
                    ref = g["%s_linear_w%d" % (key, q)]
                    assert abs(fn(sim) - ref) <= 1e-6 * abs(ref), (key, q)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_not_converged_returns_last_iterate(precision, gpu_context):
    """An iteration limit below what the tolerance needs: SG_ERR_NOT_CONVERGED (NotConverged), and
    without raising, the last iterate (its FP64-true residual below the start's) and converged = 0."""
    from smuthi_gb300 import _lib
    g = gc.load("c1")
    _product_system(g, "linear", gpu_context)
    rhs = g["rhs_linear_w0"]
    prec = _lib.SG_FP64 if precision == "fp64" else _lib.SG_FP32 | _lib.SG_DF64
    with pytest.raises(_lib.NotConverged) as e:
        gpu_context.gmres(rhs, rhs, 1e-13, restart=5, maxiter=3, precision=prec)
    assert e.value.code == _lib.SG_ERR_NOT_CONVERGED
    x, info = gpu_context.gmres(rhs, np.zeros_like(rhs), 1e-13, restart=5, maxiter=3, precision=prec,
                                raise_on_failure=False)
    assert info.converged == 0
    r = float(gpu_context.true_residual(rhs, x)[0])
    assert 1e-13 < r < 1.0 and info.max_rel_residual > 1e-13
