"""Benchmark: seconds per right-hand side to an FP64-true relative residual of 1e-6.

One "step" is one batched solve of ``--nrhs`` plane waves on the workload's
seeded sphere ensemble with the chosen form (FP32 coupling operator inside
FP64 iterative refinement, lockstep multi-RHS GMRES, all on the device),
inputs resident in HBM. The plain FP64 drop-in (FP64 operator, scipy-style
GMRES(20) with x0 = b, one RHS) is timed on the same GPU and reported beside
it. ``e2e`` repeats the chosen-form step through the public C ABI with host
(pinned) buffers, host<->device copies inside the timed region.

At one GPU the line also carries a ``target`` block: the 10 000-sphere film (16 plane waves) solved
once with the chosen form and once (first wave) with the plain FP64 drop-in, in the same run
(``--target none`` skips it; it takes several minutes, most of them in the plain FP64 solve).

``--impl reference`` times the reference's CPU path (the oracle restatement
of ``CouplingMatrixRadialLookupCPU``) on a bounded sample of the same
workload and extrapolates to seconds per RHS. Multi-GPU runs (torchrun) are
independent replicas: every rank solves its own batch, time is the max over
ranks and the value is aggregate seconds per RHS.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "s per RHS to FP64 rel. residual 1e-6: mixed+batched+learned vs plain FP64, 1 GB300"
UNIT = "s/RHS"
TOL = 1e-6
# FP64 operator applications of the plain FP64 GMRES(20) solve (x0 = b, tol 1e-6) measured with the
# plain drop-in on the same seeded workloads; the CPU reference runs the same algorithm in FP64.
PLAIN_FP64_MATVECS = {"c1": 12, "c2": 18, "c3": 17, "c4": 15, "c5": 253}


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def aggregate_max(value, world):
    """Max of a float over ranks (identity for one process)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ----------------------------------------------------------------------------------------- workload
def make_workload(name, nrhs, seed=0, n_spheres=None):
    from smuthi_gb300 import fields as flds, initial_field as init, layers, particles, workloads
    spec = workloads.build(workloads.scaled(name, n_spheres) if n_spheres else name, seed=seed)
    lm = spec["l_max"]
    parts = [particles.Sphere(position=list(p), refractive_index=spec["n_particle"], radius=spec["radius"], l_max=lm,
                              m_max=lm) for p in spec["positions"]]
    ls = layers.LayerSystem(*spec["layers"])
    wl = spec["wavelength"]
    kp = flds.reasonable_Sommerfeld_kpar_contour(wl, layer_refractive_indices=ls.refractive_indices)
    waves = list(spec["plane_waves"])
    extra = workloads.plane_waves(("random", nrhs), seed)
    waves = (waves + extra)[:nrhs]
    pos = np.array([p.position for p in parts])
    for p in parts:
        p.t_matrix = p.compute_t_matrix(wl, ls.refractive_indices[ls.layer_number(p.position[2])])
    tdiag = np.diag(parts[0].t_matrix)
    rhs = []
    for (polar, az, pol) in waves:
        a = init.PlaneWave(wl, polar, az, pol).swe_coefficients(pos, ls, lm, lm)
        rhs.append((a * tdiag[None, :]).ravel())
    return dict(spec=spec, parts=parts, ls=ls, wl=wl, kpar=kp, waves=waves,
                rhs=np.ascontiguousarray(np.stack(rhs, axis=1)))


def algorithmic_flops(n, bs, kind, nrhs):
    """Per coupling-kernel launch: interpolation once per element plus a complex MAC per RHS."""
    c_int = 4 if kind == "linear" else 12
    return float(n) * n * bs * bs * (c_int + 8 * nrhs)


def algorithmic_bytes(n, bs, kind, n_int, nrhs, fp32):
    coef = (2 if kind == "linear" else 4) * n_int * bs * bs * (8 if fp32 else 16)
    pairs = n * n * 16 if fp32 else n * 16
    vec = 3 * n * bs * nrhs * 16  # x read, y written, v read by the fused master epilogue
    return float(coef + pairs + vec)


# ----------------------------------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self, device):
        import tempfile
        self.path = os.path.join(os.environ.get("SG_CLOCK_LOG_DIR", tempfile.gettempdir()),
                                 "clocks_bench_%d.csv" % os.getpid())
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(device), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------------------- our arm
def run_ours(args, rank, world, local_rank):
    import torch
    from smuthi_gb300 import _lib
    from smuthi_gb300.linearsystem import linear_system as lsm

    torch.cuda.set_device(local_rank)
    wl = make_workload(args.workload, args.nrhs)
    spec = wl["spec"]
    t0 = time.time()
    ctx = _lib.Context(local_rank)
    W = lsm.CouplingMatrixRadialLookupCUDA(wl["wl"], wl["parts"], wl["ls"], k_parallel=wl["kpar"],
                                           resolution=spec["resolution"], interpolator_kind=spec["kind"],
                                           context=ctx)
    lsm.MasterMatrix(lsm.TMatrix(wl["parts"]), W)
    n, bs, R = spec["n_spheres"], W.blocksize, args.nrhs
    prec = _lib.SG_FP32 | (_lib.SG_DF64 if args.residual == "df64" else 0)
    pname = None
    if args.precond != "none":
        from smuthi_gb300 import learned
        cand = "precond_%s" % args.workload if args.precond == "auto" else args.precond
        if os.path.exists(os.path.join(learned.DATA_DIR, cand + ".npz")):
            pname = cand
            learned.attach(ctx, np.array([p.position[:2] for p in wl["parts"]]), bs, learned.load_params(cand, bs),
                           k=learned.load_meta(cand)["k"])
            prec |= _lib.SG_PRECOND
        elif args.precond != "auto":
            raise SystemExit("no shipped preconditioner weights named %r" % cand)
    prep_s = time.time() - t0
    n_int = W.lookup_table.shape[0] - 1
    rhs = wl["rhs"]
    dev = torch.device("cuda", local_rank)
    b_dev = torch.from_numpy(rhs).to(dev)
    x_dev = torch.zeros_like(b_dev)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # 256 MB > 129 MB L2

    def step():
        x_dev.zero_()
        return ctx.gmres_dev(b_dev.data_ptr(), x_dev.data_ptr(), R, TOL, restart=args.restart, maxiter=0,
                             precision=prec, stream=sp)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    # timed region: K batched solves, each bracketed by CUDA events on the launching stream, L2 flushed between
    barrier(world)
    clocks = ClockSampler(local_rank)
    ctx.profile(True)
    ctx.kernel_timing(reset=True)
    launches0 = ctx.launch_count()
    times, infos = [], []
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        e0.record(stream)
        info = step()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        times.append(e0.elapsed_time(e1) / 1e3)
        infos.append(info.as_dict())
    launches = ctx.launch_count() - launches0
    ms32, n32 = ctx.kernel_timing(_lib.SG_FP32, reset=False)
    msdf, ndf = ctx.kernel_timing(_lib.SG_DF64, reset=False)
    ms64, n64 = ctx.kernel_timing(_lib.SG_FP64, reset=True)
    ctx.profile(False)
    clk = clocks.stop()
    barrier(world)
    step_s = aggregate_max(float(np.sum(times)) / args.steps, world)
    value = step_s / (R * world)
    # the solution must meet the FP64-true tolerance (checked independently)
    xs = x_dev.cpu().numpy()
    relres = ctx.true_residual(rhs, np.ascontiguousarray(xs))
    assert float(relres.max()) <= TOL * 1.0001, relres.max()

    # plain FP64 drop-in: one RHS, GMRES(20), x0 = b, FP64 operator
    b0 = torch.from_numpy(np.ascontiguousarray(rhs[:, 0])).to(dev)
    x0 = b0.clone()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    ctx.profile(True)
    e0.record(stream)
    pinfo = ctx.gmres_dev(b0.data_ptr(), x0.data_ptr(), 1, TOL, restart=20, maxiter=0, precision=_lib.SG_FP64,
                          stream=sp)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    plain_s = e0.elapsed_time(e1) / 1e3
    pms64, pn64 = ctx.kernel_timing(_lib.SG_FP64, reset=True)
    ctx.profile(False)

    # e2e through the public C ABI with pinned host buffers
    hb = torch.from_numpy(rhs).pin_memory()
    hx = torch.zeros_like(hb).pin_memory()
    e2e_times = []
    for _ in range(max(1, min(args.steps, 3))):
        hx.zero_()
        torch.cuda.synchronize(dev)
        t = time.perf_counter()
        _, einfo = ctx.gmres(hb.numpy(), hx.numpy(), TOL, restart=args.restart, precision=prec,
                             raise_on_failure=True)
        e2e_times.append(time.perf_counter() - t)
    e2e_value = aggregate_max(float(np.mean(e2e_times)), world) / (R * world)

    # roofline of the dominant kernel in the timed region
    peak32 = ctx.fma_peak(_lib.SG_FP32)
    peak64 = ctx.fma_peak(_lib.SG_FP64)
    fp32_dominant = ms32 >= max(ms64, msdf)
    kind = spec["kind"]
    if fp32_dominant:
        avg_ms = ms32 / max(n32, 1)
        fl = algorithmic_flops(n, bs, kind, R)
        v32, t32 = ctx.fp32_autotune(R)[:2]
        name = {0: "coupling_kernel<float> (per receiver, RHS tile %d)" % t32,
                1: "bucket_kernel (interval-bucketed)",
                2: "sym_kernel (pair-symmetric, one warp per receiver, RHS tile %d)" % t32,
                3: "sym_kernel (pair-symmetric, two warps per receiver, RHS tile %d)" % t32,
                4: "tc_coupling_kernel (tcgen05 3xTF32, %d RHS)" % t32,
                5: "tcsym_kernel (pair-symmetric tcgen05 3xTF32, %d RHS)" % t32}.get(v32, "FP32 operator")
        peak, bound = peak32, "fp32"
        byts = algorithmic_bytes(n, bs, kind, n_int, R, True)
    elif msdf >= ms64:
        # double-float kernel on the FP32 pipe: FP64-grade flops against the FP32 pipe's peak
        avg_ms = msdf / max(ndf, 1)
        fl = algorithmic_flops(n, bs, kind, R)
        peak, bound, name = peak32, "fp32", "coupling_kernel<df64>"
        byts = algorithmic_bytes(n, bs, kind, n_int, R, False)
    else:
        avg_ms = ms64 / max(n64, 1)
        fl = algorithmic_flops(n, bs, kind, R)
        peak, bound, name = peak64, "fp64", "coupling_kernel<double>"
        byts = algorithmic_bytes(n, bs, kind, n_int, R, False)
    achieved = fl / (avg_ms * 1e-3) / 1e12
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    traffic = None
    try:
        tr = json.load(open(os.path.join(ROOT, "profiles", "ncu_traffic.json")))
        ent = tr.get("%s/%s/R%d/%s" % (args.workload, kind, R, bound))
        if ent:
            traffic = float(ent["bytes_per_launch"])
    except Exception:
        pass
    plain_avg64 = pms64 / max(pn64, 1)
    roof = {"bound": bound, "kernel": name, "achieved": round(achieved, 3), "peak": round(peak, 3),
            "unit": "TFLOP/s", "frac": round(achieved / peak, 4), "traffic": traffic,
            "peak_source": "FMA-chain probe kernel of this library, measured in this run (the pipe has no "
                           "entry in MEASURED_PEAKS.json)",
            "flops_per_launch": fl, "avg_launch_ms": round(avg_ms, 4),
            "launches": n32 if fp32_dominant else (ndf if name.endswith("<df64>") else n64),
            "hbm": {"achieved_gbs": round(byts / (avg_ms * 1e-3) / 1e9, 1), "peak_gbs": hbm_peak,
                    "frac": round(byts / (avg_ms * 1e-3) / 1e9 / hbm_peak, 4), "algorithmic_bytes": byts,
                    "peak_source": "MEASURED_PEAKS.json" if peaks else "fallback"}}
    fp64_plain_roof = {"kernel": "coupling_kernel<double> (plain drop-in, R=1)", "avg_launch_ms": round(plain_avg64, 3),
                       "achieved": round(algorithmic_flops(n, bs, kind, 1) / (plain_avg64 * 1e-3) / 1e12, 3),
                       "peak": round(peak64, 3), "unit": "TFLOP/s",
                       "frac": round(algorithmic_flops(n, bs, kind, 1) / (plain_avg64 * 1e-3) / 1e12 / peak64, 4)}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(wl, W, args.workload, pinfo.fp64_matvecs, budget_s=args.cpu_seconds)
    line = {
        "metric": METRIC, "value": round(value, 6), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(step_s * 1e3, 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32 operator; df64 (FP64-grade) residuals; fp64 refinement+Arnoldi; c128 I/O",
        "data": "synthetic seeded RSA sphere ensemble (no public dataset for this path)",
        "config": {"workload": args.workload, "n_spheres": n, "blocksize": bs, "unknowns": n * bs,
                   "nrhs": R, "interpolation": kind, "lookup_resolution_nm": spec["resolution"],
                   "restart": args.restart, "tolerance": TOL, "parallelism": "replicas" if world > 1 else "1 GPU",
                   "l2": "256 MB buffer written between timed steps (L2 is 129 MB); per-step working set "
                         "(tables, pair table, Krylov basis) also exceeds L2"},
        "plain_fp64": {"s_per_rhs": round(plain_s, 4), "iterations": pinfo.iterations,
                       "fp64_matvecs": pinfo.fp64_matvecs, "rel_residual": pinfo.max_rel_residual,
                       "restart": 20, "x0": "b"},
        "speedup_vs_plain_fp64": round(plain_s / value, 2),
        "chosen_form": {"iterations": infos[-1]["iterations"], "fp64_matvecs": infos[-1]["fp64_matvecs"],
                        "fp32_matvecs": infos[-1]["fp32_matvecs"], "refinement_steps": infos[-1]["restarts"],
                        "max_rel_residual_fp64": float(relres.max()), "learned_preconditioner": pname,
                        "precond_fallbacks": infos[-1]["precond_fallbacks"],
                        "residual_arithmetic": args.residual,
                        "batched": True, "x0": "0",
                        "fp32_kernel": dict(zip(("variant", "rhs_tile", "ms_per_receiver", "ms_bucketed", "ms_symmetric",
                                                 "ms_tensor_core", "ms_tensor_core_symmetric"), ctx.fp32_autotune(R))),
                        "fp32_kernel_variants": "0 = per-receiver, 1 = interval-bucketed, 2 = pair-symmetric (one warp per "
                                                "receiver), 3 = pair-symmetric (two warps per receiver), 4 = tensor "
                                                "cores (tcgen05 3xTF32), 5 = pair-symmetric tensor cores; RHS tile "
                                                "autotuned"},
        "prep_s": round(prep_s, 2),
        "e2e": {"value": round(e2e_value, 6), "unit": UNIT, "h2d_bytes_per_step": int(2 * rhs.nbytes),
                "d2h_bytes_per_step": int(rhs.nbytes)},
        "gpu_launches": int(launches),
        "roofline": roof,
        "plain_fp64_kernel": fp64_plain_roof,
        "residual_kernel": {"kernel": "coupling_kernel<%s> (true residual, %d RHS)" % (args.residual, R),
                            "avg_launch_ms": round((msdf / max(ndf, 1)) if ndf else (ms64 / max(n64, 1)), 3),
                            "launches": ndf if ndf else n64},
        "clocks": clk,
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    table = PLAIN_FP64_MATVECS.get(args.workload)
    line["plain_fp64"]["matvecs_used_by_reference_arm"] = table
    line["plain_fp64"]["reference_arm_count_consistent"] = table == pinfo.fp64_matvecs
    ctx.close()
    if world == 1 and args.target != "none":
        line["target"] = run_target(args, local_rank)
    return line


# ----------------------------------------------------------------------------------------- target
def run_target(args, local_rank):
    """The target configuration measured once in the same run: the chosen form on the 10 000-sphere film
    (16 plane waves) against the plain FP64 drop-in on its first wave, both to an FP64-true relative
    residual of 1e-6 on the same GPU. Warm-up: one application of every operator the solves use (the
    pair table, the double-float coefficients, the FP32 autotuning and the preconditioner's near-field
    blocks are built on first use); the timed solves then run once each (a chosen-form solve takes
    minutes, the plain one several)."""
    import torch
    from smuthi_gb300 import _lib, learned
    from smuthi_gb300.linearsystem import linear_system as lsm
    name = args.target
    R = 16
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    t0 = time.time()
    wl = make_workload(name, R)
    spec = wl["spec"]
    ctx = _lib.Context(local_rank)
    W = lsm.CouplingMatrixRadialLookupCUDA(wl["wl"], wl["parts"], wl["ls"], k_parallel=wl["kpar"],
                                           resolution=spec["resolution"], interpolator_kind=spec["kind"],
                                           context=ctx)
    lsm.MasterMatrix(lsm.TMatrix(wl["parts"]), W)
    n, bs = spec["n_spheres"], W.blocksize
    prec = _lib.SG_FP32 | _lib.SG_DF64
    pname = "precond_%s" % name
    if os.path.exists(os.path.join(learned.DATA_DIR, pname + ".npz")):
        learned.attach(ctx, np.array([p.position[:2] for p in wl["parts"]]), bs, learned.load_params(pname, bs),
                       k=learned.load_meta(pname)["k"])
        prec |= _lib.SG_PRECOND
    else:
        pname = None
    rhs = wl["rhs"]
    b_dev = torch.from_numpy(rhs).to(dev)
    x_dev = torch.zeros_like(b_dev)
    tmp = torch.empty_like(b_dev)
    sp = torch.cuda.current_stream(dev).cuda_stream
    for p in (_lib.SG_FP32, _lib.SG_DF64):
        ctx.master_matvec_dev(b_dev.data_ptr(), tmp.data_ptr(), R, p, stream=sp)
    if pname:
        ctx.precond_apply_dev(b_dev.data_ptr(), tmp.data_ptr(), R, stream=sp)
    torch.cuda.synchronize(dev)
    prep_s = time.time() - t0
    stream = torch.cuda.current_stream(dev)
    clocks = ClockSampler(local_rank)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    info = ctx.gmres_dev(b_dev.data_ptr(), x_dev.data_ptr(), R, TOL, restart=args.restart, maxiter=0,
                         precision=prec, stream=sp)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    chosen_s = e0.elapsed_time(e1) / 1e3
    relres = ctx.true_residual(rhs, np.ascontiguousarray(x_dev.cpu().numpy()))
    b0 = torch.from_numpy(np.ascontiguousarray(rhs[:, 0])).to(dev)
    x0 = b0.clone()
    e0.record(stream)
    pinfo = ctx.gmres_dev(b0.data_ptr(), x0.data_ptr(), 1, TOL, restart=20, maxiter=0, precision=_lib.SG_FP64,
                          stream=sp)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    plain_s = e0.elapsed_time(e1) / 1e3
    clk = clocks.stop()
    prelres = ctx.true_residual(rhs[:, 0], np.ascontiguousarray(x0.cpu().numpy()))
    out = {"workload": name, "n_spheres": n, "blocksize": bs, "unknowns": n * bs, "nrhs": R,
           "interpolation": spec["kind"],
           "chosen_form": {"s_per_rhs": round(chosen_s / R, 4), "solve_s": round(chosen_s, 3),
                           "iterations": info.iterations, "refinement_steps": info.restarts,
                           "fp32_matvecs": info.fp32_matvecs, "fp64_grade_matvecs": info.fp64_matvecs,
                           "max_rel_residual_fp64": float(relres.max()), "learned_preconditioner": pname,
                           "precond_fallbacks": info.precond_fallbacks, "residual_arithmetic": "df64",
                           "fp32_kernel": dict(zip(("variant", "rhs_tile", "ms_per_receiver", "ms_bucketed",
                                                    "ms_symmetric", "ms_tensor_core", "ms_tensor_core_symmetric"),
                                                   ctx.fp32_autotune(R)))},
           "plain_fp64": {"s_per_rhs": round(plain_s, 3), "iterations": pinfo.iterations,
                          "fp64_matvecs": pinfo.fp64_matvecs, "rel_residual_fp64": float(prelres[0]),
                          "restart": 20, "x0": "b"},
           "speedup_vs_plain_fp64": round(plain_s / (chosen_s / R), 2),
           "met": bool(relres.max() <= TOL * 1.0001 and prelres[0] <= TOL * 1.0001),
           "prep_s": round(prep_s, 1), "clocks": clk,
           "warmup": "one application of the FP32 and double-float operators and the preconditioner (one-time "
                     "set-up and autotuning); each solve timed once with CUDA events"}
    ctx.close()
    return out


# ----------------------------------------------------------------------------------------- CPU reference
def cpu_baseline(wl, W, workload, fp64_matvecs, budget_s=15.0):
    """Time the oracle restatement of CouplingMatrixRadialLookupCPU on a receiving-particle sample."""
    import oracle.physics as ophys
    import oracle.solve as osv
    parts = [ophys.Sphere(p.position, p.refractive_index, p.radius, p.l_max, p.m_max) for p in wl["parts"]]
    t_build = time.time()
    Wo = osv.RadialLookupCPU(parts, W.lookup_table, W.radial_distance_array, wl["spec"]["kind"])
    t_build = time.time() - t_build
    n = len(parts)
    bs = W.blocksize
    rng = np.random.default_rng(3)
    x = rng.standard_normal(W.shape[0]) + 1j * rng.standard_normal(W.shape[0])
    rows = 1
    elapsed = 0.0
    while True:
        sel = rng.choice(n, size=rows, replace=False)
        t = time.time()
        Wo.matvec(x, rows=sel)
        elapsed = time.time() - t
        if elapsed > budget_s / 4 or rows >= n:
            break
        rows = min(n, max(rows * 2, int(rows * budget_s / 4 / max(elapsed, 1e-3))))
    per_elem = elapsed / (rows * n * bs * bs)
    matvec_s = per_elem * n * n * bs * bs
    value = matvec_s * fp64_matvecs
    return {"value": round(value, 3), "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "oracle CouplingMatrixRadialLookupCPU matvec over %d of %d receiving particles (%.1f s), "
                      "%.1f ns/element; s/RHS = full matvec (%.1f s) x %d FP64 matvecs of the plain GMRES(20) "
                      "solve; interpolator set-up %.1f s not included" % (rows, n, elapsed, per_elem * 1e9,
                                                                          matvec_s, fp64_matvecs, t_build)}


_REF_WORKER = {}


def _ref_worker_init(parts_spec, tab, rho, kind):
    import oracle.physics as ophys
    import oracle.solve as osv
    parts = [ophys.Sphere(*p) for p in parts_spec]
    _REF_WORKER["W"] = osv.RadialLookupCPU(parts, tab, rho, kind)


def _ref_worker_rows(args):
    x, rows = args
    _REF_WORKER["W"].matvec(x, rows=rows)
    return len(rows)


def run_reference(args, rank, world):
    if rank != 0:
        return None
    import oracle.layers as olay
    import oracle.physics as ophys
    import oracle.solve as osv
    import oracle.special as osp
    from smuthi_gb300 import workloads
    spec = workloads.build(args.workload, seed=0)
    lm = spec["l_max"]
    parts = [ophys.Sphere(list(p), spec["n_particle"], spec["radius"], lm, lm) for p in spec["positions"]]
    ls = olay.LayerSystem(*spec["layers"])
    kp = osp.sommerfeld_kpar_contour(spec["wavelength"], ls.refractive_indices)
    tab, rho = ophys.radial_coupling_lookup_table(spec["wavelength"], parts, ls, kp, spec["resolution"])
    n = len(parts)
    bs = tab.shape[1]
    rng = np.random.default_rng(3)
    x = rng.standard_normal(n * bs) + 1j * rng.standard_normal(n * bs)
    fp64_matvecs = PLAIN_FP64_MATVECS.get(args.workload, 20)
    # the reference's CPU matvec is single-threaded numpy/scipy per receiving row: spread the sampled
    # rows over every host core with one process each (spawned: nothing here touches the GPU)
    import multiprocessing as mp
    cores = max(1, min(os.cpu_count() or 1, 64))
    rows = max(1, int(args.ref_rows)) * cores
    parts_spec = [(list(p.position), p.refractive_index, p.radius, p.l_max, p.m_max) for p in parts]
    ctx_mp = mp.get_context("spawn")
    vals = []
    with ctx_mp.Pool(cores, initializer=_ref_worker_init, initargs=(parts_spec, tab, rho, spec["kind"])) as pool:
        pool.map(_ref_worker_rows, [(x, np.array([0]))] * cores)  # every worker has built its interpolators
        for i in range(args.warmup + args.steps):
            sel = rng.choice(n, size=rows, replace=False)
            chunks = [c for c in np.array_split(sel, cores) if len(c)]
            t = time.time()
            pool.map(_ref_worker_rows, [(x, c) for c in chunks])
            el = time.time() - t
            if i >= args.warmup:
                vals.append(el / (rows * n * bs * bs) * n * n * bs * bs * fp64_matvecs)
    v = float(np.mean(vals))
    return {"impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128 (FP64)", "data": "synthetic seeded RSA sphere ensemble",
            "config": {"workload": args.workload, "n_spheres": n, "blocksize": bs, "interpolation": spec["kind"],
                       "nrhs": 1},
            "cpu_baseline": {"value": round(v, 3), "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "per step: oracle CouplingMatrixRadialLookupCPU matvec over %d receiving "
                                       "particles of %d on %d processes, extrapolated to the full matvec x %d "
                                       "FP64 matvecs of GMRES(20)" % (rows, n, cores, fp64_matvecs)},
            "e2e": {"value": round(v, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5"])
    ap.add_argument("--nrhs", type=int, default=16)
    ap.add_argument("--restart", type=int, default=64)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-rows", type=int, default=4)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precond", default="auto",
                    help="learned-preconditioner weights name, 'none', or 'auto' (precond_<workload> if shipped)")
    ap.add_argument("--residual", default="df64", choices=["df64", "fp64"],
                    help="arithmetic of the refinement's true residuals")
    ap.add_argument("--target", default="c5", choices=["c5", "c3", "c2", "none"],
                    help="configuration of the one-shot target block (1 GPU only): chosen form vs plain FP64")
    args = ap.parse_args(argv)
    rank, world, local_rank = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="nccl" if args.impl == "ours" else "gloo")
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    else:
        if rank == 0:
            from smuthi_gb300.build import build
            build()
        barrier(world)
        line = run_ours(args, rank, world, local_rank)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
