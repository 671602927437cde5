"""Benchmark: solves/sec to eps=1e-4 on one GB300, batched FP32 SPOCK vs plain FP64 SPOCK.

Workload (one "step"): the uniform batch of 1,024 instances that share the config-2 problem
(3-state Markov chain, N=10, stopping stage 4 -> 607 nodes; nx=50, nu=20; quadratic-plus-linear
costs, box constraints, AVaR(0.95)), each with its own x0 ~ U[-1,1]^50, solved by SuperMann
(Anderson memory 5) to tol 1e-4 (absolute and relative, CacheBuilder::tol).  Synthetic data
from fixed seeds; the per-instance vectors of the batch (11 GB) are far larger than L2.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the CPU FP64 implementation of the same iteration (the oracle's C
restatement of the reference solver; the reference's own solver is CUDA code that needs the
unavailable GPUtils library) on all host threads over a bounded sample per step.
Prints one JSON line (rank 0).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "spock.cu_gb300"))

METRIC = "solves/sec to eps=1e-4 on one GB300 (batched+warm-start FP32 vs plain FP64 SPOCK)"
PROBLEM_DIR = os.environ.get("SPOCK_BENCH_DIR", "/tmp/spock_bench")
TOL, ANDERSON = 1e-4, 5


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=1024)
    ap.add_argument("--max-iters", type=int, default=20000)
    ap.add_argument("--seed", type=int, default=0)
    return ap.parse_args()


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def workload(seed, count, rank=0):
    from spock_gb300 import configs
    path, x0 = configs.cached("config2", PROBLEM_DIR + f"_r{rank}", seed=seed, count=count + 64 * rank)
    return path, np.ascontiguousarray(x0[64 * rank:64 * rank + count])


def config_dict(batch, world):
    return {"workload": "config4-uniform: %d instances of config2 (Markov 3 states, N=10, stopping 4, 607 nodes, "
                        "nx=50, nu=20, quadratic-plus-linear costs, box |x|<=3 |u|<=1, AVaR 0.95), eps=1e-4, "
                        "Anderson memory 5" % batch,
            "instances_per_gpu": batch, "precision": "fp32 iteration, fp64 controller",
            "l2": "inputs larger than L2 (per-step working set ~11 GB)", "parallelism": f"replicas x{world}"}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.proc = None
        self.index = index
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_{index}.csv") if os.path.isdir(os.path.join(ROOT, "gpurun_out")) \
            else f"/tmp/spock_clocks_{index}.csv"

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        self.proc.wait()
        self.fh.close()
        sm, mx, reasons = [], 0., set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample(path, x0s, threads, iters):
    """Oracle (FP64 C) on `threads` threads, each instance stopped after `iters` outer SPOCK
    iterations; returns seconds per outer iteration per instance."""
    from oracle import oracle
    oracle.build()
    P = oracle.Problem(path)
    opts = oracle.options(tol=TOL, anderson=ANDERSON, max_iters=iters)
    secs, status, its, _, _ = P.solve_many(np.repeat(x0s[:1], threads, axis=0) if len(x0s) < threads else x0s[:threads],
                                           opts, threads)
    done = float(np.sum(np.maximum(its, 1)))
    return secs * threads / done, secs


def measured_cpu_iterations():
    """Outer iterations per config-2 solve measured by full oracle solves (committed summary)."""
    fn = os.path.join(ROOT, "profiles", "cpu_oracle_config2.md")
    if os.path.exists(fn):
        for line in open(fn):
            if line.startswith("mean_outer_iterations:"):
                return float(line.split(":")[1])
    return None


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    path, x0s = workload(args.seed, max(threads, 1))
    iters = 25
    per_iter = []
    for _ in range(args.warmup):
        cpu_sample(path, x0s, threads, iters)
    t_total = 0.
    for _ in range(args.steps):
        spi, secs = cpu_sample(path, x0s, threads, iters)
        per_iter.append(spi)
        t_total += secs
    spi = statistics.median(per_iter)
    it_solve = measured_cpu_iterations() or float(args.max_iters)
    value = threads / (spi * it_solve)
    sample = (f"{threads} instances on {threads} threads, {iters} outer SPOCK iterations each per step; "
              f"solves/s = threads / (s per outer iteration x {it_solve:.0f} outer iterations per solve, "
              f"measured by full FP64 solves)")
    out = {"metric": METRIC, "value": value, "unit": "solves/s", "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_total / max(args.steps, 1),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded)", "config": config_dict(args.batch, world),
           "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def run_gpu(args):
    import torch
    import spock_gb300 as sg
    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    sg.build()
    B = args.batch
    path, x0s = workload(args.seed, B, rank)
    tree = sg.ScenarioTree(path)
    data = sg.ProblemData(tree)
    cache = (sg.CacheBuilder(tree, data).tol(TOL).andersonBuffer(ANDERSON).maxIters(args.max_iters)
             .precision(32).batch(B).device(local).build())
    nx = tree.numStates()
    x0_dev = torch.tensor(x0s.T.copy(), dtype=torch.float32, device=f"cuda:{local}").contiguous()  # [nx][B]

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    def device_step():
        st = cache.solveDevice(x0_dev.data_ptr())
        return st

    for _ in range(args.warmup):
        torch.cuda.synchronize()
        device_step()
    clocks = Clocks(local)
    barrier()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record()
    statuses, iters, rounds, launches = [], [], 0, 0
    for _ in range(args.steps):
        st = device_step()
        statuses.append(st)
        iters.append(cache.solveIters())
        r, l = cache.runStats()
        rounds += r
        launches += l
    e1.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    t_dev = ms / 1e3
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([t_dev])
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_dev = float(tt[0])
    st_all = np.concatenate(statuses)
    it_all = np.concatenate(iters)
    conv = st_all == 0
    value = B * world * args.steps / t_dev

    # end to end through the public API: host x0 in, statuses + first inputs out
    barrier()
    t1 = time.perf_counter()
    for _ in range(args.steps):
        cache.runSpockBatch(x0s)
        u0 = cache.firstInputs()
    barrier()
    t_e2e = time.perf_counter() - t1
    e2e = {"value": B * world * args.steps / t_e2e, "unit": "solves/s",
           "h2d_bytes_per_step": int(B * nx * 4), "d2h_bytes_per_step": int(B * (tree.numInputs() * 4 + 4 + 4))}

    # roofline of the dominant kernel: CUDA-event time of single launches on the engine stream
    per_round = {}
    for k in ["lstar", "lop", "mlstar", "mlop", "dyn", "reduce", "update"]:
        kms, kbytes = cache.kernelTime(k, 10)
        per_round[k] = (kms, kbytes)
    dom = max(per_round, key=lambda k: per_round[k][0])
    kms, kbytes = per_round[dom]
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        peak, peak_src = float(peaks["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        peak, peak_src = 6800., "fallback"
    achieved = kbytes / (kms / 1e3) / 1e9
    traffic = None
    fn = os.path.join(ROOT, "profiles", "traffic.md")
    if os.path.exists(fn):
        for line in open(fn):
            if line.startswith(f"{dom}_bytes_per_launch:"):
                traffic = float(line.split(":")[1])

    cpu = None
    if rank == 0:
        threads = os.cpu_count() or 1
        spi, _ = cpu_sample(path, x0s, threads, 25)
        mean_it = float(np.mean(it_all[conv])) if conv.any() else float(args.max_iters)
        cpu_val = threads / (spi * mean_it)
        cpu = {"value": cpu_val, "unit": "solves/s", "cores": threads, "kind": "port",
               "sample": f"{threads} instances x 25 outer SPOCK iterations (FP64 C oracle, {threads} threads); "
                         f"extrapolated with the {mean_it:.0f} outer iterations per solve of this run"}
    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
               "config": config_dict(B, world),
               "e2e": e2e,
               "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                            "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                            "peak_source": peak_src, "kernel_ms": kms, "algorithmic_bytes": kbytes,
                            "per_kernel_ms": {k: v[0] for k, v in per_round.items()}},
               "cpu_baseline": cpu, "clocks": clk, "gpu_launches": int(launches),
               "converged": int(conv.sum()), "instances": int(st_all.size),
               "outer_iterations": {"mean": float(np.mean(it_all)), "max": int(np.max(it_all))},
               "rounds_per_step": rounds / args.steps, "wall_s": wall}
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
