"""Benchmark: solves/sec to eps=1e-4 on one GB300, batched warm-started FP32 SPOCK vs plain FP64 SPOCK.

Workload: the uniform batch of 1,024 instances sharing the config-2 problem (3-state Markov
chain, N=10, stopping stage 4 -> 607 nodes; nx=50, nu=20; quadratic-plus-linear costs Q=diag
U[1,10], R=diag U[0.1,1], q, r ~ N(0,1); box |x|<=3, |u|<=1; AVaR(0.95)), with every cost term
multiplied by 1e-3 (same minimiser; at the literal scale the cost-to-go is near 800 and SPOCK
stalls near a residual of 1e-2 in FP64 as in FP32).  Each instance has its own x0 ~ U[-1,1]^50.

One step is one receding-horizon re-solve of the whole batch: every x0 moves by a disturbance
U[-0.05, 0.05]^50 (clipped to [-1, 1]) and every instance is re-solved by SuperMann (Anderson
memory 5) to tol(1e-4) -- absolute and relative tolerance 1e-4, CacheBuilder::tol -- warm-started
from its previous solution (the previousSolution path of cache.cuh:611-632), which stays on the
device.  Before the warm-up steps the batch is solved once from a cold start (not timed).
Synthetic data from fixed seeds; the batch's per-instance vectors (~10 GB) are far larger than L2.

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
TOL, ANDERSON, COST_SCALE, DRIFT = 1e-4, 5, 1e-3, 0.05


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=1024)
    ap.add_argument("--max-iters", type=int, default=20000)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-fp64-baseline", action="store_true", help="skip the plain FP64 SPOCK solves on the GPU")
    return ap.parse_args()


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def instance_slice(count, rank):
    """Replicas: rank r solves its own instances r*count .. (r+1)*count-1 (no data exchange)."""
    return slice(rank * count, (rank + 1) * count)


def max_over_ranks(seconds, world):
    """The job's time: the slowest rank's (a gloo or NCCL all-reduce when world > 1)."""
    if world <= 1:
        return float(seconds)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(seconds)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t[0])


def workload(seed, count, rank=0):
    """Problem folder and this rank's initial states."""
    from spock_gb300 import configs
    path, x0 = configs.cached("config2", PROBLEM_DIR, seed=seed, count=count * (rank + 1), cost_scale=COST_SCALE)
    return path, np.ascontiguousarray(x0[instance_slice(count, rank)])


def trajectory(x0s, steps, seed, rank=0):
    """Initial states of the successive re-solves: x_k = clip(x_{k-1} + U[-0.05, 0.05], -1, 1)."""
    rng = np.random.default_rng(1000003 * (seed + 1) + rank)
    out, x = [], x0s.copy()
    for _ in range(steps):
        x = np.clip(x + rng.uniform(-DRIFT, DRIFT, x.shape), -1., 1.)
        out.append(np.ascontiguousarray(x))
    return out


def config_dict(batch, world):
    return {"workload": "config4-uniform: %d instances of config2 (Markov 3 states, N=10, stopping 4, 607 nodes, "
                        "nx=50, nu=20, quadratic-plus-linear costs x 1e-3, box |x|<=3 |u|<=1, AVaR 0.95); step = "
                        "warm-started re-solve of every instance after an x0 disturbance U[-0.05,0.05]^50, "
                        "tol(1e-4), Anderson memory 5" % batch,
            "instances_per_gpu": batch, "precision": "fp32 iteration, fp64 controller and reductions",
            "cost_scale": COST_SCALE, "tolerance": "CacheBuilder::tol(1e-4): absolute and relative",
            "l2": "inputs larger than L2 (per-step working set ~10 GB)", "parallelism": f"replicas x{world}"}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        import tempfile
        self.proc = None
        self.index = index
        self.path = os.path.join(tempfile.gettempdir(), f"spock_clocks_{os.getpid()}_{index}.csv")

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


def cpu_resolves(path, x0_steps, z_start, threads, max_iters):
    """FP64 oracle re-solves on `threads` host threads, one instance each: instance i starts from
    z_start[i] and is re-solved along x0_steps[k][i] (each re-solve warm-started from the last).
    z_start (C-contiguous float64, count x size) is updated in place to the last solutions.
    Returns (wall seconds per step, statuses, mean T evaluations) over the steps."""
    from oracle import oracle
    oracle.build()
    P = oracle.Problem(path)
    opts = oracle.options(tol=TOL, anderson=ANDERSON, max_iters=max_iters)
    zs = z_start
    secs, sts, calls = [], [], []
    for x in x0_steps:
        t, st, its, c, _ = P.solve_many_warm(x, zs, opts, threads, warm=True)
        secs.append(t)
        sts.append(st)
        calls.append(c)
    if not secs:
        return secs, np.zeros(0, dtype=np.int32), 0.
    return secs, np.concatenate(sts), float(np.mean(np.concatenate(calls)))


def cpu_cold(path, x0s, threads, max_iters):
    """FP64 oracle cold solves (one instance per thread); returns the solutions (count x size)."""
    from oracle import oracle
    oracle.build()
    P = oracle.Problem(path)
    opts = oracle.options(tol=TOL, anderson=ANDERSON, max_iters=max_iters)
    zs = np.zeros((x0s.shape[0], P.size))
    P.solve_many_warm(x0s, zs, opts, threads, warm=False)
    return zs


def run_reference(args):
    """The CPU implementation of the same iteration (the oracle's FP64 C restatement of the
    reference solver), timed on every host thread: one instance per thread, solved cold (not
    timed), then W warm-up and K timed receding-horizon re-solves along the benchmark's x0
    trajectory, each warm-started from the instance's previous solution."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n = min(threads, args.batch)
    path, x0s = workload(args.seed, args.batch)
    traj = [x[:n] for x in trajectory(x0s, args.warmup + args.steps, args.seed)]
    zs = cpu_cold(path, x0s[:n], n, args.max_iters)
    cpu_resolves(path, traj[:args.warmup], zs, n, args.max_iters)
    secs, st, calls = cpu_resolves(path, traj[args.warmup:], zs, n, args.max_iters)
    total = float(np.sum(secs))
    value = n * args.steps / total
    sample = (f"{n} instances on {n} threads (one each), FP64 C oracle; per step every instance is re-solved to "
              f"tol(1e-4) warm-started from its previous solution; {int((st == 0).sum())}/{st.size} converged, "
              f"{calls:.0f} T evaluations per re-solve")
    out = {"metric": METRIC, "value": value, "unit": "solves/s", "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / max(args.steps, 1),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded)", "config": config_dict(args.batch, world),
           "cpu_baseline": {"value": value, "unit": "solves/s", "cores": n, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def fp64_cold_gpu(path, x0s, device, count, max_iters):
    """Plain cold-started FP64 SPOCK on the same GPU, one instance at a time (the reference's usage,
    examples/random/main.cu:41-70): solves/s over `count` solves."""
    import spock_gb300 as sg
    tree = sg.ScenarioTree(path)
    data = sg.ProblemData(tree)
    c = (sg.CacheBuilder(tree, data).tol(TOL).andersonBuffer(ANDERSON).maxIters(max_iters)
         .precision(64).batch(1).device(device).build())
    c.runSpock(x0s[0])  # warm-up: graph capture, autotuning
    t0 = time.perf_counter()
    st, its = [], []
    for k in range(count):
        c.reset()
        st.append(c.runSpock(x0s[k]))
        its.append(c.solveIter())
    el = time.perf_counter() - t0
    return {"value": count / el, "unit": "solves/s", "solves": count, "converged": int(sum(s == 0 for s in st)),
            "outer_iterations_mean": float(np.mean(its)), "seconds": el,
            "note": "cold FP64 solves stop at tol(1e-4)'s relative tolerance (about 1e-3 here)"}


# DRAM bytes (read + write) of one launch of a kernel, from an ncu capture (dram__bytes_read.sum +
# dram__bytes_write.sum) of this workload: {(kernel, batch): bytes}.  The bench reports it as
# roofline.traffic when the dominant kernel and batch have an entry.
TRAFFIC_BYTES = {}


def fp64_error(z_gpu, z_ref, nu, scaling_u, size_prim, nodes):
    """Error of the GPU's FP32 solutions against the FP64 oracle's solutions of the same instances
    (same x0, same warm start, same tolerance): relative error of the optimal cost s_0 (the root's
    s, the first entry of the primal s block) and max error of the unscaled first inputs u_0."""
    oS = size_prim - nodes
    cost_g, cost_r = z_gpu[:, oS], z_ref[:, oS]
    u_g, u_r = z_gpu[:, :nu] / scaling_u, z_ref[:, :nu] / scaling_u
    return {"cost_rel_err_max": float(np.max(np.abs(cost_g - cost_r) / np.maximum(np.abs(cost_r), 1e-30))),
            "cost_rel_err_mean": float(np.mean(np.abs(cost_g - cost_r) / np.maximum(np.abs(cost_r), 1e-30))),
            "u0_abs_err_max": float(np.max(np.abs(u_g - u_r))),
            "u0_rel_err_max": float(np.max(np.abs(u_g - u_r)) / max(np.max(np.abs(u_r)), 1e-30))}


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

    def fp32_cache():
        return (sg.CacheBuilder(tree, data).tol(TOL).andersonBuffer(ANDERSON).maxIters(args.max_iters)
                .precision(32).batch(B).device(local).build())
    cache = fp32_cache()
    snap = fp32_cache()  # holds the iterate the timed steps start from, for the end-to-end replay
    nx, nu = tree.numStates(), tree.numInputs()
    extra = 2  # untimed steps after the timed ones: GPU against the FP64 oracle on the same re-solves
    traj = trajectory(x0s, args.warmup + args.steps + extra, args.seed, rank)
    x_dev = [torch.tensor(x.T.copy(), dtype=torch.float32, device=f"cuda:{local}").contiguous() for x in traj]
    threads = os.cpu_count() or 1
    sample = np.linspace(0, B - 1, min(threads, B)).astype(int)  # instances the CPU legs re-solve

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    cache.runSpockBatch(x0s)  # the cold solve the receding-horizon loop starts from (not timed)
    cold_conv = int((cache.statuses() == 0).sum())
    for k in range(args.warmup):
        cache.resolveDevice(x_dev[k].data_ptr())
    snap.copyIterateFrom(cache)
    clocks = Clocks(local)
    barrier()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record()
    statuses, iters, calls, rounds, launches = [], [], [], 0, 0
    for k in range(args.steps):
        st = cache.resolveDevice(x_dev[args.warmup + k].data_ptr())
        statuses.append(st)
        cnt = cache.countersAll()
        iters.append(cnt[:, 6].copy())
        calls.append(cnt[:, 5].copy())
        r, l = cache.runStats()
        rounds += r
        launches += l
    e1.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    t_dev = max_over_ranks(e0.elapsed_time(e1) / 1e3, world)
    st_all, it_all, calls_all = np.concatenate(statuses), np.concatenate(iters), np.concatenate(calls)
    conv = st_all == 0
    value = B * world * args.steps / t_dev

    # end to end through the public API on the same steps: the iterate the timed steps started
    # from is put back (not timed), then every step copies host x0 in (double) and reads the
    # statuses, iterations and first inputs back
    cache.copyIterateFrom(snap)
    barrier()
    t1 = time.perf_counter()
    st_e2e = []
    for k in range(args.steps):
        st_e2e.append(cache.resolveBatch(traj[args.warmup + k]))
        u0 = cache.firstInputs()
    barrier()
    t_e2e = max_over_ranks(time.perf_counter() - t1, world)
    e2e = {"value": B * world * args.steps / t_e2e, "unit": "solves/s",
           "h2d_bytes_per_step": int(B * nx * 8), "d2h_bytes_per_step": int(B * (nu * 8 + 4 + 8)),
           "same_steps_as_value": True, "converged": int((np.concatenate(st_e2e) == 0).sum())}
    del snap

    # the same re-solves on the GPU (FP32) and in the FP64 oracle on the host cores: `extra` more
    # steps, each instance of the sample starting from the GPU's solution of the step before
    z_gpu, z_cpu, cpu_secs, cpu_st, cpu_calls = [], [], [], [], []
    for k in range(extra):
        x_next = traj[args.warmup + args.steps + k]
        z_before = np.stack([cache.solution(int(b)) for b in sample]) if rank == 0 else None
        cache.resolveBatch(x_next)
        if rank == 0:
            z_gpu.append(np.stack([cache.solution(int(b)) for b in sample]))
            secs, cst, ccalls = cpu_resolves(path, [x_next[sample]], z_before, len(sample), args.max_iters)
            z_cpu.append(z_before)  # updated in place to the oracle's solutions
            cpu_secs += secs
            cpu_st.append(cst)
            cpu_calls.append(ccalls)

    # roofline of the dominant kernel: CUDA-event time of single launches on the solver stream
    per_kernel = {}
    for k in ["lstar", "lop", "mlstar", "mlop", "dyn", "reduce", "update"]:
        per_kernel[k] = cache.kernelTime(k, 10)
    dom = max(per_kernel, key=lambda k: per_kernel[k][0])
    kms, kbytes = per_kernel[dom]
    try:
        peak, peak_src = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        peak, peak_src = 6800., "fallback"
    achieved = kbytes / (kms / 1e3) / 1e9
    traffic = TRAFFIC_BYTES.get((dom, B))

    out = None
    if rank == 0:
        # CPU baseline: the FP64 oracle's re-solves of the sample above, one instance per thread
        n = len(sample)
        cst = np.concatenate(cpu_st)
        cpu = {"value": n * len(cpu_secs) / float(np.sum(cpu_secs)), "unit": "solves/s", "cores": n, "kind": "port",
               "sample": f"{n} instances x {len(cpu_secs)} warm re-solves of this workload (each from the GPU's "
                         f"solution of the step before), FP64 C oracle, one instance per thread; "
                         f"{int((cst == 0).sum())}/{cst.size} converged, {np.mean(cpu_calls):.0f} T evaluations "
                         f"per re-solve"}
        err = fp64_error(np.concatenate(z_gpu), np.concatenate(z_cpu), nu, data.scaling()[nx:nx + nu],
                         cache.sizePrimal(), tree.numNodes())
        err.update({"instances": int(cst.size), "reference": "FP64 oracle (CPU): same x0, same warm start, same "
                    "tol(1e-4)", "reference_converged": int((cst == 0).sum())})
        fp64 = None if args.no_fp64_baseline else fp64_cold_gpu(path, x0s, local, 16, args.max_iters)
        out = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
               "config": config_dict(B, world), "e2e": e2e,
               "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak, "traffic": traffic, "peak_source": peak_src,
                            "kernel_ms": kms, "algorithmic_bytes": kbytes,
                            "per_kernel_ms": {k: v[0] for k, v in per_kernel.items()},
                            "per_kernel_gbs": {k: v[1] / v[0] / 1e6 for k, v in per_kernel.items()}},
               "cpu_baseline": cpu, "clocks": clk, "gpu_launches": int(launches), "fp64_error": err,
               "converged": int(conv.sum()), "instances": int(st_all.size), "cold_start_converged": cold_conv,
               "outer_iterations": {"mean": float(np.mean(it_all)), "max": int(np.max(it_all))},
               "t_evaluations_mean": float(np.mean(calls_all)), "rounds_per_step": rounds / args.steps,
               "tuning": cache.tuning(), "fp64_cold_single_gpu": fp64, "wall_s": wall}
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
