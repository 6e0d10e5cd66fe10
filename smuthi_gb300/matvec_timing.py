"""Time the master operator y = x - T W x of a workload shape at one arithmetic.

    python -m smuthi_gb300.matvec_timing --workload c2 --nrhs 16 --precision df64 --repeat 3

Builds the seeded sphere ensemble of the shape, applies the operator ``repeat`` times to the
plane-wave right-hand sides (device buffers, the context's stream) and prints one JSON line with
the mean CUDA-event time per launch.

    python -m smuthi_gb300.matvec_timing --volume --n-spheres 1000 --nrhs 16 --precision fp64 --kind linear

times the volume-lookup operator instead: spheres (radius 60 nm) on a jittered 200 nm square
lattice at seeded heights in [100, 160] nm above a glass substrate, 550 nm, 10 nm lookup grid. It is also the small, fixed launch sequence used to profile
one coupling kernel: the first operator application carries one-time set-up (pair table, double-float
coefficients, FP32 kernel autotuning), the later ones are steady state.

    python -m smuthi_gb300.matvec_timing --nearfield 16384 --repeat 3

times the electric field of a seeded upgoing plane-wave expansion (550 nm in air above glass, the
default Sommerfeld contour and azimuth grid) at that many points above the particles' plane, host
copies included (`sg_pwe_field`).
"""
import argparse
import json

import numpy as np

from . import _lib, learned

PRECISIONS = {"fp64": _lib.SG_FP64, "fp32": _lib.SG_FP32, "df64": _lib.SG_DF64, "tf32x3": _lib.SG_TF32X3}


def volume_system(n, nrhs, kind, seed=0):
    """Spheres at different heights above a substrate with the GPU volume lookup (see module doc)."""
    from . import fields as flds
    from . import layers, particles
    from .linearsystem import linear_system as lsm
    rng = np.random.default_rng(seed)
    side = int(np.ceil(np.sqrt(n)))
    cells = np.array([(a, b) for a in range(side) for b in range(side)][:n], dtype=float)
    xy = 200.0 * cells + rng.uniform(-20.0, 20.0, size=cells.shape)
    z = rng.uniform(100.0, 160.0, size=n)
    parts = [particles.Sphere(position=[x, y, zz], refractive_index=2.0 + 0.02j, radius=60.0, l_max=3, m_max=3)
             for (x, y), zz in zip(xy, z)]
    ls = layers.LayerSystem([0, 0], [1.52, 1])
    wl = 550.0
    kp = flds.reasonable_Sommerfeld_kpar_contour(wl, layer_refractive_indices=ls.refractive_indices)
    ctx = _lib.Context(0)
    W = lsm.CouplingMatrixVolumeLookupCUDA(wl, parts, ls, k_parallel=kp, resolution=10.0, interpolator_kind=kind,
                                           context=ctx)
    for p in parts:
        p.t_matrix = p.compute_t_matrix(wl, ls.refractive_indices[ls.layer_number(p.position[2])])
    lsm.MasterMatrix(lsm.TMatrix(parts), W)
    rhs = rng.standard_normal((W.shape[0], nrhs)) + 1j * rng.standard_normal((W.shape[0], nrhs))
    return dict(ctx=ctx, n=n, blocksize=W.blocksize, rhs=rhs,
                table_shape=list(W.lookup_table_plus.shape))


def nearfield_timing(n_points, repeat, seed=0):
    """Seconds per electric-field evaluation of a seeded plane-wave expansion at n_points (see above)."""
    import time
    from . import fields as flds
    from . import layers
    from .fields.expansions import PlaneWaveExpansion
    rng = np.random.default_rng(seed)
    ls = layers.LayerSystem([0, 0], [1.52, 1])
    wl = 550.0
    kp = flds.reasonable_Sommerfeld_kpar_contour(wl, layer_refractive_indices=ls.refractive_indices)
    az, _ = flds.angular_arrays(np.pi / 360)
    k = flds.angular_frequency(wl)
    pwe = PlaneWaveExpansion(k, kp, az, kind='upgoing', reference_point=[0, 0, 100.0], lower_z=100.0)
    pwe.coefficients = rng.standard_normal((2, len(kp), len(az))) + 1j * rng.standard_normal((2, len(kp), len(az)))
    x, y = rng.uniform(-2000, 2000, n_points), rng.uniform(-2000, 2000, n_points)
    z = rng.uniform(300, 1000, n_points)
    ctx = _lib.Context(0)
    pwe.electric_field(x, y, z, context=ctx)  # warm-up
    t = time.perf_counter()
    for _ in range(repeat):
        pwe.electric_field(x, y, z, context=ctx)
    dt = (time.perf_counter() - t) / repeat
    ctx.close()
    return {"nearfield_points": n_points, "k_parallel_nodes": len(kp), "azimuths": len(az), "seconds": dt,
            "ns_per_point_and_node": dt / (n_points * len(kp) * len(az)) * 1e9}


def main(argv=None):
    import torch
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--workload", default="c2")
    ap.add_argument("--n-spheres", type=int, default=None)
    ap.add_argument("--nrhs", type=int, default=16)
    ap.add_argument("--precision", default="df64", choices=sorted(PRECISIONS))
    ap.add_argument("--repeat", type=int, default=3)
    ap.add_argument("--volume", action="store_true", help="time the volume lookup (particles at different heights)")
    ap.add_argument("--kind", default="linear", choices=("linear", "cubic", "cubic_hermite"))
    ap.add_argument("--nearfield", type=int, default=0, metavar="POINTS",
                    help="time the near field of a plane-wave expansion at this many points instead")
    ap.add_argument("--fp32-kernel", default=None, metavar="VARIANT:TILE",
                    help="fix the FP32 kernel (0 per-receiver, 1 bucketed, 2 pair-symmetric, 3 pair-symmetric "
                         "with two warps per receiver, 4 tensor cores, 5 pair-symmetric tensor cores, tile = nrhs "
                         "for 4 and 5) and its RHS tile "
                         "instead of the autotuner's choice")
    a = ap.parse_args(argv)
    if a.nearfield:
        print(json.dumps(nearfield_timing(a.nearfield, a.repeat)))
        return
    if a.volume:
        system = volume_system(a.n_spheres or 1000, a.nrhs, a.kind)
    else:
        system = learned.film_system(a.workload, a.n_spheres, nrhs=a.nrhs)
    ctx = system["ctx"]
    dev = torch.device("cuda", ctx.device)
    x = torch.from_numpy(np.ascontiguousarray(system["rhs"])).to(dev)
    y = torch.empty_like(x)
    prec = PRECISIONS[a.precision]
    if a.fp32_kernel:
        v, t = (int(s) for s in a.fp32_kernel.split(":"))
        ctx.fp32_set_kernel(a.nrhs, v, t)
    ctx.master_matvec_dev(x.data_ptr(), y.data_ptr(), a.nrhs, prec)  # set-up and warm-up
    torch.cuda.synchronize(dev)
    ctx.profile(True)
    ctx.kernel_timing(reset=True)
    for _ in range(a.repeat):
        ctx.master_matvec_dev(x.data_ptr(), y.data_ptr(), a.nrhs, prec)
    ms, n = ctx.kernel_timing(prec, reset=True)
    ctx.profile(False)
    out = {"workload": "volume/" + a.kind if a.volume else a.workload, "n_spheres": system["n"],
           "blocksize": system["blocksize"], "nrhs": a.nrhs, "precision": a.precision, "launches": n,
           "ms_per_launch": ms / max(n, 1)}
    if a.volume:
        out["table_shape"] = system["table_shape"]
    if a.precision == "fp32" and not a.volume:
        out["fp32_kernel"] = dict(zip(("variant", "rhs_tile", "ms_per_receiver", "ms_bucketed", "ms_symmetric",
                                       "ms_tensor_core", "ms_tensor_core_symmetric"),
                                      ctx.fp32_autotune(a.nrhs)))
    print(json.dumps(out))
    ctx.close()


if __name__ == "__main__":
    main()
