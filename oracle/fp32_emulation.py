"""Warm re-solves of the benchmark workload under the oracle's FP32 emulation modes.

    python oracle/fp32_emulation.py [--instances 8] [--modes gpu_fp32,...]
    python oracle/fp32_emulation.py --cold --tol 1e-5 --max-iters 5000 [--instances 8]

Test infrastructure (it runs the oracle only): it explains how single-precision arithmetic
changes the SPOCK iteration's path.  The workload is the benchmark's (config 2 with costs
x 1e-3, tol 1e-4, Anderson memory 5): `--instances` initial states are solved cold and
re-solved once in plain FP64, then re-solved a second time along the benchmark's x0 trajectory
under each mode, starting from the same FP64 iterates.  Prints one JSON line per mode with the
mean / max T evaluations and outer iterations of that re-solve.  With --cold, each mode instead
solves the instances from a cold start to tol(--tol) within --max-iters outer iterations.
"""
import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# this folder on sys.path would make `oracle` resolve to oracle/oracle.py instead of the package
sys.path = [ROOT, os.path.join(ROOT, "spock.cu_gb300")] + [p for p in sys.path if os.path.abspath(p or ".") != HERE]

from oracle import oracle as O  # noqa: E402

MODES = {
    "fp64": 0,
    "data_fp32": O.EMU_DATA,
    "data_acc_fp32": O.EMU_DATA | O.EMU_ACC,
    "gpu_fp32": O.EMU_GPU_FP32,
    "gpu_fp32_fwd64": O.EMU_GPU_FP32 | O.EMU_FWD64,
    "gpu_fp32_fwd_dot2": O.EMU_GPU_FP32 | O.EMU_FWDC,
    "gpu_fp32_fwd_dot2_states": O.EMU_GPU_FP32 | O.EMU_FWDCX,
    "gpu_fp32_fwd_kahan": O.EMU_GPU_FP32 | O.EMU_FWDK,
}


def main():
    import bench
    ap = argparse.ArgumentParser()
    ap.add_argument("--instances", type=int, default=8)
    ap.add_argument("--modes", default=",".join(MODES))
    ap.add_argument("--cold", action="store_true")
    ap.add_argument("--tol", type=float, default=bench.TOL)
    ap.add_argument("--max-iters", type=int, default=20000)
    args = ap.parse_args()
    n = args.instances
    path, x0s = bench.workload(0, n)
    traj = bench.trajectory(x0s, 2, 0)
    opts = O.options(tol=args.tol, anderson=bench.ANDERSON, max_iters=args.max_iters)
    O.set_emulation(0)
    P = O.Problem(path)
    zs = np.zeros((n, P.size))
    if not args.cold:
        P.solve_many_warm(x0s[:n], zs, opts, n, warm=False)
        P.solve_many_warm(traj[0][:n], zs, opts, n, warm=True)
    for name in args.modes.split(","):
        O.set_emulation(MODES[name])
        Pm = O.Problem(path)  # loaded under the mode (OR_EMU_DATA rounds the problem data)
        z = zs.copy()
        if args.cold:
            secs, st, its, calls, _ = Pm.solve_many_warm(x0s[:n], z, opts, n, warm=False)
        else:
            secs, st, its, calls, _ = Pm.solve_many_warm(traj[1][:n], z, opts, n, warm=True)
        print(json.dumps({"mode": name, "flags": MODES[name], "instances": n, "start": "cold" if args.cold else "warm",
                          "tol": args.tol, "converged": int((st == 0).sum()),
                          "T_evaluations_mean": float(calls.mean()), "T_evaluations_max": int(calls.max()),
                          "outer_iterations_mean": float(its.mean()), "outer_iterations_max": int(its.max()),
                          "seconds": round(secs, 1)}), flush=True)
    O.set_emulation(0)


if __name__ == "__main__":
    main()
