"""Time the master operator y = x - T W x of a workload shape at one arithmetic.

    python -m smuthi_gb300.matvec_timing --workload c2 --nrhs 16 --precision df64 --repeat 3

Builds the seeded sphere ensemble of the shape, applies the operator ``repeat`` times to the
plane-wave right-hand sides (device buffers, the context's stream) and prints one JSON line with
the mean CUDA-event time per launch. It is also the small, fixed launch sequence used to profile
one coupling kernel: the first operator application carries one-time set-up (pair table, double-float
coefficients, FP32 kernel autotuning), the later ones are steady state.
"""
import argparse
import json

import numpy as np

from . import _lib, learned

PRECISIONS = {"fp64": _lib.SG_FP64, "fp32": _lib.SG_FP32, "df64": _lib.SG_DF64, "tf32x3": _lib.SG_TF32X3}


def main(argv=None):
    import torch
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--workload", default="c2")
    ap.add_argument("--n-spheres", type=int, default=None)
    ap.add_argument("--nrhs", type=int, default=16)
    ap.add_argument("--precision", default="df64", choices=sorted(PRECISIONS))
    ap.add_argument("--repeat", type=int, default=3)
    a = ap.parse_args(argv)
    system = learned.film_system(a.workload, a.n_spheres, nrhs=a.nrhs)
    ctx = system["ctx"]
    dev = torch.device("cuda", ctx.device)
    x = torch.from_numpy(np.ascontiguousarray(system["rhs"])).to(dev)
    y = torch.empty_like(x)
    prec = PRECISIONS[a.precision]
    ctx.master_matvec_dev(x.data_ptr(), y.data_ptr(), a.nrhs, prec)  # set-up and warm-up
    torch.cuda.synchronize(dev)
    ctx.profile(True)
    ctx.kernel_timing(reset=True)
    for _ in range(a.repeat):
        ctx.master_matvec_dev(x.data_ptr(), y.data_ptr(), a.nrhs, prec)
    ms, n = ctx.kernel_timing(prec, reset=True)
    ctx.profile(False)
    print(json.dumps({"workload": a.workload, "n_spheres": system["n"], "blocksize": system["blocksize"],
                      "nrhs": a.nrhs, "precision": a.precision, "launches": n, "ms_per_launch": ms / max(n, 1)}))
    ctx.close()


if __name__ == "__main__":
    main()
