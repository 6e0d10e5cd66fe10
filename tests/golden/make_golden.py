"""Generate golden fixtures by running the reference SMUTHI code itself.

Run where the reference source tree is available, naming it in ``SMUTHI_REFERENCE_ROOT``::

    SMUTHI_REFERENCE_ROOT=/root/reference python tests/golden/make_golden.py [case ...]

The reference is imported with the three test-only shims of ``refload.py``.
Each case writes ``tests/golden/<case>.npz`` with the inputs (geometry,
optics, Sommerfeld contour), the reference's lookup table (whole, or a row
subset plus checksums for larger cases), T-matrices, initial-field
coefficients, right-hand side, coupling and master matvecs of a seeded
vector, GMRES solutions and the extinction / total scattering cross
sections. Package versions are recorded in every file.
"""
import os
import sys
import time

import numpy as np
import scipy
import sympy

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import refload  # noqa: E402
from smuthi_gb300 import workloads  # noqa: E402

CASES = {
    # the reference radial-lookup unit-test geometry (tests/unit_tests/multiple_scattering_tests/
    # test_radial_lookup.py:31-37): mixed m_max, lossy film; excited by a plane wave
    "wg3": dict(custom="wg3", kinds=("linear", "cubic"), full_table=True, solve_kinds=("linear", "cubic")),
    "c1": dict(shape="c1", n=100, kinds=("linear", "cubic"), full_table=False, solve_kinds=("linear",)),
    "c2s": dict(shape="c2", n=120, kinds=("cubic",), full_table=False, solve_kinds=("cubic",)),
    "c3s": dict(shape="c3", n=40, kinds=("cubic",), full_table=False, solve_kinds=("cubic",)),
    "c5s": dict(shape="c5", n=60, kinds=("linear",), full_table=False, solve_kinds=("linear",)),
    # particles at different heights above a substrate: the reference takes its volume lookup
    # (CouplingMatrixVolumeLookupCPU, linear_system.py:592-667) with 2-D (rho, z1 +- z2) tables
    "vol5": dict(custom="vol5", kinds=("linear", "cubic"), full_table=False, solve_kinds=("linear", "cubic"),
                 volume=True, near_field=True),
}
# plane-wave expansions with seeded coefficients, evaluated by the reference's CPU field code
# (smuthi/fields/expansions.py:635-900, cpu_precision='double precision')
PWE_CASES = ("pwe1",)
PARITY_TOL = 1e-13


def _geometry(case, part, lay, init):
    if case.get("custom") == "wg3":
        spheres = [dict(position=[0, 0, 150], refractive_index=2.4 + 0.1j, radius=100, l_max=3, m_max=3),
                   dict(position=[102, -100, 150], refractive_index=1.9 + 0.2j, radius=80, l_max=3, m_max=2),
                   dict(position=[202, 100, 150], refractive_index=1.7 + 0.0j, radius=90, l_max=3, m_max=3)]
        layers = ([0, 400, 0], [1.5, 2 + 0.01j, 1])
        wl = 550.0
        waves = [(np.pi * 7 / 8, np.pi / 3, 0)]
        resolution = 5.0
        contour = dict(neff_waypoints=[0, 0.5, 0.8 - 0.01j, 2 - 0.01j, 2.5, 5], neff_resolution=1e-2)
        ref_point = [200, 200, 200]
    elif case.get("custom") == "vol5":
        spheres = [dict(position=[0, 0, 100], refractive_index=2.0 + 0.05j, radius=70, l_max=3, m_max=3),
                   dict(position=[190, 40, 130], refractive_index=2.0 + 0.05j, radius=70, l_max=3, m_max=3),
                   dict(position=[-60, 200, 90], refractive_index=1.8 + 0.0j, radius=60, l_max=3, m_max=2),
                   dict(position=[250, 280, 160], refractive_index=2.0 + 0.05j, radius=70, l_max=3, m_max=3),
                   dict(position=[-230, -150, 120], refractive_index=2.0 + 0.05j, radius=70, l_max=3, m_max=3)]
        layers = ([0, 0], [1.52, 1])
        wl = 550.0
        waves = [(np.pi, 0.0, 0), (np.pi * 5 / 6, 0.7, 1)]
        resolution = 10.0
        contour = dict()
        ref_point = [0, 0, 0]
    else:
        spec = workloads.scaled(case["shape"], case["n"])
        spec = workloads.build(spec, seed=0)
        spheres = [dict(position=list(p), refractive_index=spec["n_particle"], radius=spec["radius"],
                        l_max=spec["l_max"], m_max=spec["l_max"]) for p in spec["positions"]]
        layers = spec["layers"]
        wl = spec["wavelength"]
        waves = spec["plane_waves"]
        if case["shape"] == "c5":
            waves = [waves[0], (np.pi / 5, 1.0, 1)]
        resolution = spec["resolution"]
        contour = dict()
        ref_point = [0, 0, 0]
    return spheres, layers, wl, waves, resolution, contour, ref_point


def run_case(name, case):
    sm = refload.import_reference()
    import smuthi.fields as flds
    import smuthi.initial_field as init
    import smuthi.layers as lay
    import smuthi.linearsystem.linear_system as lsm
    import smuthi.particles as part
    import smuthi.postprocessing.far_field as ff
    import smuthi.simulation as simul

    spheres, layers, wl, waves, resolution, contour, ref_point = _geometry(case, part, lay, init)
    out = dict(positions=np.array([s["position"] for s in spheres], float),
               radii=np.array([s["radius"] for s in spheres], float),
               n_particle=np.array([s["refractive_index"] for s in spheres], complex),
               l_max=np.array([s["l_max"] for s in spheres]), m_max=np.array([s["m_max"] for s in spheres]),
               thicknesses=np.array(layers[0], float), layer_n=np.array(layers[1], complex),
               wavelength=wl, waves=np.array(waves, float), resolution=resolution,
               wave_reference_point=np.array(ref_point, float),
               neff_waypoints=np.array(contour.get("neff_waypoints", []), complex),
               neff_resolution=contour.get("neff_resolution", 1e-2),
               versions=np.array(["numpy " + np.__version__, "scipy " + scipy.__version__,
                                  "sympy " + sympy.__version__, "smuthi " + sm.__version__]))
    rng = np.random.Generator(np.random.PCG64(1234))

    for kind in case["kinds"]:
        for iw, (polar, az, pol) in enumerate(waves):
            if iw > 0 and kind != case["kinds"][0]:
                continue
            plist = [part.Sphere(**s) for s in spheres]
            ls = lay.LayerSystem(list(layers[0]), list(layers[1]))
            pw = init.PlaneWave(vacuum_wavelength=wl, polar_angle=polar, azimuthal_angle=az, polarization=int(pol),
                                amplitude=1, reference_point=ref_point)
            tol = PARITY_TOL if kind in case["solve_kinds"] else 1.0
            sim = simul.Simulation(layer_system=ls, particle_list=plist, initial_field=pw, solver_type='gmres',
                                   solver_tolerance=tol, store_coupling_matrix=False,
                                   coupling_matrix_lookup_resolution=resolution,
                                   coupling_matrix_interpolator_kind=kind, log_to_terminal=False, **contour)
            t0 = time.time()
            sim.run()
            t_run = time.time() - t0
            lsys = sim.linear_system
            cm = lsys.coupling_matrix
            volume = case.get("volume", False)
            assert type(cm).__name__ == ('CouplingMatrixVolumeLookupCPU' if volume else
                                         'CouplingMatrixRadialLookupCPU')
            tag = "%s_w%d" % (kind, iw)
            if iw == 0:
                if volume and "kpar" not in out:
                    out["kpar"] = np.array(flds.default_Sommerfeld_k_parallel_array)
                    out["rho_grid"] = cm.rho_array
                    out["sz_grid"] = cm.sum_z_array
                    out["dz_grid"] = cm.diff_z_array
                    for key, tab in (("plus", cm.lookup_table_plus), ("minus", cm.lookup_table_minus)):
                        out["table_%s_dtype" % key] = np.array(str(tab.dtype))
                        out["table_%s_shape" % key] = np.array(tab.shape)
                        rows = np.unique(np.concatenate([np.arange(0, 8), rng.choice(len(tab), size=6,
                                                                                   replace=False)]))
                        out["table_%s_rows" % key] = rows
                        out["table_%s_subset" % key] = tab[rows]
                        out["table_%s_abs_sum" % key] = np.abs(tab.astype(complex)).sum()
                        wts = np.cos(0.37 * np.arange(tab.size)).reshape(tab.shape)
                        out["table_%s_weighted_sum" % key] = (tab.astype(complex) * wts).sum()
                    out["t_diag"] = np.concatenate([np.diag(p.t_matrix) for p in plist])
                if "kpar" not in out:
                    out["kpar"] = np.array(flds.default_Sommerfeld_k_parallel_array)
                    out["rho_grid"] = cm.radial_distance_array
                    tab = cm.lookup_table
                    out["table_shape"] = np.array(tab.shape)
                    if case["full_table"]:
                        out["table"] = tab
                    else:
                        rows = np.unique(np.concatenate([np.arange(0, min(48, len(tab))),
                                                         rng.choice(len(tab), size=12, replace=False)]))
                        out["table_rows"] = rows
                        out["table_subset"] = tab[rows]
                    out["table_abs_sum"] = np.abs(tab).sum()
                    wts = np.cos(0.37 * np.arange(tab.size)).reshape(tab.shape)
                    out["table_weighted_sum"] = (tab * wts).sum()
                    out["t_diag"] = np.concatenate([np.diag(p.t_matrix) for p in plist])
                x = rng.standard_normal(cm.shape[0]) + 1j * rng.standard_normal(cm.shape[0])
                out["x_" + kind] = x
                out["Wx_" + kind] = cm.linear_operator.matvec(x)
                out["Mx_" + kind] = lsys.master_matrix.linear_operator.matvec(x)
            out["a_" + tag] = np.concatenate([p.initial_field.coefficients for p in plist])
            out["rhs_" + tag] = lsys.t_matrix.right_hand_side()
            if kind in case["solve_kinds"]:
                b = np.concatenate([p.scattered_field.coefficients for p in plist])
                out["b_" + tag] = b
                mres = lsys.master_matrix.linear_operator.matvec(b) - out["rhs_" + tag]
                out["relres_" + tag] = np.linalg.norm(mres) / np.linalg.norm(out["rhs_" + tag])
                t1 = time.time()
                out["sigma_ext_" + tag] = ff.extinction_cross_section(sim)
                out["sigma_sca_" + tag] = ff.total_scattering_cross_section(sim)
                print("  %s: run %.1fs, cross sections %.1fs, relres %.2e, ext %.6e sca %.6e"
                      % (tag, t_run, time.time() - t1, out["relres_" + tag], out["sigma_ext_" + tag],
                         out["sigma_sca_" + tag]), flush=True)
                if case.get("near_field") and tag == case["kinds"][0] + "_w0":
                    # scattered field above the particles from its plane-wave expansion in the top layer
                    # (smuthi/postprocessing/scattered_field.py:80-150)
                    import smuthi.postprocessing.scattered_field as sf
                    i_top = ls.number_of_layers() - 1
                    pu, pd = sf.scattered_field_pwe(wl, plist, ls, i_top)
                    pts = np.stack([np.linspace(-300, 400, 6), np.linspace(250, -150, 6),
                                    np.linspace(320, 520, 6)], axis=1)
                    out["nf_points"] = pts
                    out["nf_azimuthal_angles"] = np.array(pu.azimuthal_angles)
                    out["nf_kpar"] = np.array(pu.k_parallel)
                    for nm, pwe in (("up", pu), ("down", pd)):
                        e = pwe.electric_field(pts[:, 0], pts[:, 1], pts[:, 2], cpu_precision='double precision')
                        out["nf_E_" + nm] = np.array(e)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path) // 1024, "KiB", flush=True)


def run_pwe_case(name):
    """Seeded PlaneWaveExpansion objects (complex contour, both kinds) and their E and H fields."""
    refload.import_reference()
    import smuthi.fields as flds
    import smuthi.fields.expansions as fldex
    rng = np.random.Generator(np.random.PCG64(77))
    wl = 550.0
    k = flds.angular_frequency(wl) * (1.3 + 0.02j)
    kpar = flds.reasonable_Sommerfeld_kpar_contour(wl, layer_refractive_indices=[1.3 + 0.02j, 1.0],
                                                    neff_resolution=2e-2)
    alpha = np.linspace(0, 2 * np.pi, 37)
    pts = np.stack([rng.uniform(-400, 400, 9), rng.uniform(-400, 400, 9), rng.uniform(-50, 350, 9)], axis=1)
    out = dict(wavelength=wl, k=k, kpar=kpar, alpha=alpha, points=pts,
               versions=np.array(["numpy " + np.__version__, "scipy " + scipy.__version__]))
    for kind, ref, lo, hi in (("upgoing", [10.0, -20.0, 30.0], 0.0, np.inf),
                              ("downgoing", [-15.0, 5.0, 250.0], -np.inf, 300.0)):
        pwe = fldex.PlaneWaveExpansion(k=k, k_parallel=kpar, azimuthal_angles=alpha, kind=kind,
                                       reference_point=ref, lower_z=lo, upper_z=hi)
        decay = np.exp(-np.abs(kpar) / abs(k))[None, :, None]
        pwe.coefficients = decay * (rng.standard_normal(pwe.coefficients.shape)
                                    + 1j * rng.standard_normal(pwe.coefficients.shape))
        out["g_" + kind] = pwe.coefficients
        out["ref_" + kind] = np.array(ref)
        out["bounds_" + kind] = np.array([lo, hi])
        out["E_" + kind] = np.array(pwe.electric_field(pts[:, 0], pts[:, 1], pts[:, 2],
                                                       cpu_precision='double precision'))
        out["H_" + kind] = np.array(pwe.magnetic_field(pts[:, 0], pts[:, 1], pts[:, 2], wl,
                                                       cpu_precision='double precision'))
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path) // 1024, "KiB", flush=True)


def main(argv):
    names = argv or list(CASES) + list(PWE_CASES)
    for n in names:
        print("case", n, flush=True)
        if n in PWE_CASES:
            run_pwe_case(n)
        else:
            run_case(n, CASES[n])


if __name__ == "__main__":
    main(sys.argv[1:])
