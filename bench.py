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
    ap.add_argument("--fp64-finish", type=int, default=0,
                    help="rounds after which the last <= 32 running instances of a step finish in FP64 (0: never)")
    ap.add_argument("--study", choices=["warmstart", "precision", "mixed", "finish"],
                    help="instead of the benchmark line: the learned warm start (config 5), the precision study "
                         "(config 3), the mixed batch (config 4 mixed) or the FP64 finish thresholds "
                         "(--finish-rounds) on the benchmark's steps; one JSON line per result")
    ap.add_argument("--finish-rounds", default="0,400,800,1600", help="finish: FP64-finish thresholds to time")
    ap.add_argument("--train", type=int, default=16384, help="warmstart: training solves")
    ap.add_argument("--pca-rows", type=int, default=8192, help="warmstart: solutions the PCA basis is fitted on")
    ap.add_argument("--train-tol", type=float, default=1e-4, help="warmstart: tolerance of the training solves")
    ap.add_argument("--test", type=int, default=10240, help="warmstart: held-out initial states")
    ap.add_argument("--epochs", type=int, default=40, help="warmstart: MLP training epochs")
    ap.add_argument("--variants", default="ball,box", help="precision: config-3 input constraints to run (ball, box)")
    ap.add_argument("--kernels", help="instead of the benchmark line: comma-separated round kernels (lstar, lop, "
                                      "mlstar, mlop, dyn, reduce, update, round) timed one launch at a time on a "
                                      "random iterate of --batch instances, tiles 1 per CTA (profiling driver)")
    ap.add_argument("--kernel-reps", type=int, default=5, help="kernels: timed launches after one untimed")
    ap.add_argument("--gemm", action="store_true", help="instead of the benchmark line: the tensor-core GEMM at the "
                                                        "warm start's reconstruction shape and an MLP shape")
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


def config_dict(batch, world, finish=0):
    prec = "fp32 iteration, fp64 controller and reductions"
    if finish > 0:
        prec += f"; after {finish} rounds the last <= 32 running instances finish in fp64"
    return {"workload": "config4-uniform: %d instances of config2 (Markov 3 states, N=10, stopping 4, 607 nodes, "
                        "nx=50, nu=20, quadratic-plus-linear costs x 1e-3, box |x|<=3 |u|<=1, AVaR 0.95); step = "
                        "warm-started re-solve of every instance after an x0 disturbance U[-0.05,0.05]^50, "
                        "tol(1e-4), Anderson memory 5" % batch,
            "instances_per_gpu": batch, "precision": prec, "fp64_finish_rounds": finish,
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


# DRAM bytes (read + write) of one launch of a kernel (the dynamics sweep: of one sweep), from an
# ncu capture (dram__bytes_read.sum + dram__bytes_write.sum) of this workload at 256 instances,
# scaled to 1,024 by the instances (node matrices counted once): {(kernel, batch): bytes}.  The
# bench reports it as roofline.traffic when the dominant kernel and batch have an entry.
TRAFFIC_BYTES = {("dyn", 1024): 666e6, ("update", 1024): 8.90e9, ("reduce", 1024): 4.57e9}


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
    if args.fp64_finish > 0:
        cache.fp64Finish(args.fp64_finish)
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
               "config": config_dict(B, world, args.fp64_finish), "e2e": e2e,
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


def study_warmstart(args):
    """Learned warm start on the benchmark's problem family (config 5 at a stated scale): train
    data = cold FP32 batch solves of x0 ~ U[-1, 1]^50 at tol(--train-tol); PCA(128) of the first
    --pca-rows solutions; MLP 50 -> 1024 -> 1024 -> 128 (the library's tensor-core kernels) on
    the coefficients of all of them; then --test held-out x0 in batches of 1,024 solved to the
    absolute tolerance 1e-4 (a warm start's initial error is small, so tol(1e-4) decides by its
    absolute part; the cold comparison is held to the same absolute tolerance) from: a cold
    start, the learned start, and the previous held-out instance's solution (the shifted
    previous solution of a stream of requests).  Prints one JSON line per phase and method."""
    import torch
    import spock_gb300 as sg
    from spock_gb300.warmstart import PcaMlpWarmStart
    sg.build()
    B = 1024
    path, _ = workload(args.seed, 1)
    t = sg.ScenarioTree(path)
    d = sg.ProblemData(t)
    rng = np.random.default_rng(2026 + args.seed)
    ntr = (args.train + B - 1) // B * B
    nte = max(B, args.test // B * B)
    xtr = rng.uniform(-1., 1., (ntr, t.numStates()))
    xte = rng.uniform(-1., 1., (nte, t.numStates()))

    def cache(absolute, tol=1e-4):
        b = sg.CacheBuilder(t, d).andersonBuffer(ANDERSON).maxIters(args.max_iters).precision(32).batch(B)
        b = b.toleranceAbsolute(tol).toleranceRelative(0.) if absolute else b.tol(tol)
        return b.build()

    def emit(rec):
        print(json.dumps(rec), flush=True)

    ws = PcaMlpWarmStart(k=128, hidden=1024, seed=args.seed)
    ctr = cache(False, args.train_tol)
    t0 = time.time()
    zs, coefs, conv = [], [], 0
    for s0 in range(0, ntr, B):
        conv += int((ctr.runSpockBatch(xtr[s0:s0 + B]) == 0).sum())
        z = torch.tensor(ctr.solutions(), dtype=torch.float32, device="cuda")
        if s0 < args.pca_rows:
            zs.append(z)
            if s0 + B >= min(args.pca_rows, ntr):
                ws.fit_basis(torch.cat(zs))
                coefs += [ws.project(zz) for zz in zs]
                zs = []
        else:
            coefs.append(ws.project(z))
    emit({"study": "warmstart", "phase": "data", "solves": ntr, "converged": conv, "tol": args.train_tol,
          "seconds": round(time.time() - t0, 1), "pca_rows": min(args.pca_rows, ntr), "pca_explained": ws.explained})
    t0 = time.time()
    losses = ws.fit_mlp(xtr, torch.cat(coefs), epochs=args.epochs, batch=B, lr=1e-3)
    emit({"study": "warmstart", "phase": "fit", "seconds": round(time.time() - t0, 1), "epochs": args.epochs,
          "loss_first": losses[0], "loss_last": losses[-1]})
    methods = ("cold_tol", "cold_absolute", "learned", "shifted_previous")
    res = {m: {"seconds": 0., "iters": [], "conv": 0, "u0_err": 0., "n": 0} for m in methods}
    cc, ca, cw, cp = cache(False), cache(True), cache(True), cache(True)
    z_prev = None  # the last solution of the previous batch (instance B-1)

    def timed(name, c, f, x):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        st = f()
        res[name]["seconds"] += time.perf_counter() - t1
        res[name]["iters"].append(c.solveIters())
        res[name]["conv"] += int((st == 0).sum())
        res[name]["n"] += len(x)
        return st

    for s0 in range(0, nte, B):
        x = xte[s0:s0 + B]
        # cold, reference tolerance semantics: tol(1e-4) captures its relative part (~1e-3 here)
        timed("cold_tol", cc, lambda: cc.runSpockBatch(x), x)
        u_cold = cc.firstInputs()
        z_cold = torch.tensor(cc.solutions(), dtype=torch.float32, device="cuda")
        if s0 == 0:  # cold at the warm starts' absolute tolerance: the equal-accuracy comparison (one batch)
            timed("cold_absolute", ca, lambda: ca.runSpockBatch(x), x)
        # previous request's solution: instance i starts from instance i-1's (the first from the
        # previous batch's last)
        prev = torch.roll(z_cold, 1, 0)
        if z_prev is not None:
            prev[0] = z_prev
        z_prev = z_cold[-1].clone()
        zp = prev.T.contiguous()
        cp.setIterateDevice(zp.data_ptr(), 32)
        timed("shifted_previous", cp, lambda: cp.resolveBatch(x), x)
        timed("learned", cw, lambda: (ws.warm_start(cw, x), cw.resolveBatch(x))[1], x)  # prediction included
        for name, c in (("shifted_previous", cp), ("learned", cw)):
            res[name]["u0_err"] = max(res[name]["u0_err"], float(np.abs(c.firstInputs() - u_cold).max()))
    for name, r in res.items():
        it = np.concatenate(r["iters"])
        emit({"study": "warmstart", "method": name, "instances": r["n"], "batch": B, "converged": r["conv"],
              "solves_per_s": r["n"] / r["seconds"], "iters_mean": float(it.mean()), "iters_max": int(it.max()),
              "u0_max_diff_vs_cold_tol": r["u0_err"] if name in ("learned", "shifted_previous") else None,
              "tolerance": "tol(1e-4), relative part decides" if name == "cold_tol" else "absolute 1e-4 (relative 0)"})


def study_precision(args):
    """Config 3 (i.i.d. 5 events, N=8, stopping 3: 781 nodes; nx=100, nu=40; box on x; AVaR 0.9)
    with costs x 1e-3 (at the literal scale SPOCK stalls on this problem in FP64 too, as on
    config 2), with the input ball ||u||_2 <= 2 and with the input box |u_i| <= 2.  Eight
    initial states (32 GPU instances, rows reused) solved cold:
      * FP32 on the GPU (batched kernels) to tol(1e-4) and to tol(1e-6);
      * the FP64 oracle on the host cores to tol(1e-4) (at most 1,500 iterations, 240 s);
      * (input box) the FP64 polish on the GPU of the FP32 solution to tol(1e-6), the tight
        reference (FP64 with the input ball exceeds the kernels' shared memory at this size).
    Errors of each FP32 result against the FP64 ones: relative error of the optimal cost s_0 and
    max error of the unscaled states and inputs.  One JSON line per comparison."""
    import spock_gb300 as sg
    from oracle import oracle
    from spock_gb300 import configs
    sg.build()
    oracle.build()
    n, B = 8, 32
    for ball in [v == "ball" for v in args.variants.split(",")]:
        path, x0 = configs.cached("config3", PROBLEM_DIR, seed=args.seed, count=n, ball=ball, cost_scale=COST_SCALE)
        xb = np.resize(x0, (B, x0.shape[1]))
        t = sg.ScenarioTree(path)
        d = sg.ProblemData(t)
        P = oracle.Problem(path)
        oS = P.size_prim - P.n
        name = "config3 x 1e-3 " + ("input ball" if ball else "input box")
        t0 = time.time()
        zr = np.zeros((n, P.size))
        _, st_r, it_r, _, _ = P.solve_many_warm(x0, zr, oracle.options(tol=1e-4, anderson=ANDERSON, max_iters=1500,
                                                                       max_time=240.), n, warm=False)
        ref = {"oracle fp64 tol(1e-4)": (zr, np.array([P.states_inputs(z)[0] for z in zr]),
                                         np.array([P.states_inputs(z)[1] for z in zr]),
                                         f"{int((st_r == 0).sum())}/{n} converged, {np.mean(it_r):.0f} iterations, "
                                         f"{time.time() - t0:.0f} s on {n} threads")}

        def gpu(c):
            return (np.stack([c.solution(b) for b in range(n)]), np.stack([c.states(b) for b in range(n)]),
                    np.stack([c.inputs(b) for b in range(n)]))
        res = {}
        for eps in (1e-4, 1e-6):
            c = (sg.CacheBuilder(t, d).tol(eps).andersonBuffer(ANDERSON).maxIters(args.max_iters).precision(32)
                 .batch(B).build())
            t1 = time.time()
            c.runSpockBatch(xb)
            res[eps] = (c, time.time() - t1)
            if eps == 1e-6 and not ball:
                c64 = (sg.CacheBuilder(t, d).tol(eps).andersonBuffer(ANDERSON).maxIters(args.max_iters)
                       .precision(64).batch(B).build())
                t1 = time.time()
                st64 = c64.polish(c, xb)
                ref["gpu fp32 + fp64 polish tol(1e-6)"] = gpu(c64) + (
                    f"{int((st64[:n] == 0).sum())}/{n} converged, {np.mean(c64.solveIters()[:n]):.0f} iterations, "
                    f"{time.time() - t1:.1f} s",)
        for eps, (c, secs) in res.items():
            zg, xg, ug = gpu(c)
            for rname, (zr_, xr_, ur_, note) in ref.items():
                print(json.dumps({"study": "precision", "problem": name, "solver": f"gpu fp32 tol({eps:g})",
                                  "converged": int((c.statuses()[:n] == 0).sum()), "instances": n,
                                  "iters_mean": float(np.mean(c.solveIters()[:n])), "seconds": round(secs, 2),
                                  "against": rname, "against_run": note,
                                  "cost_rel_err_max": float(np.max(np.abs(zg[:, oS] - zr_[:, oS]) / np.abs(zr_[:, oS]))),
                                  "states_err_max": float(np.abs(xg - xr_).max()),
                                  "inputs_err_max": float(np.abs(ug - ur_).max()),
                                  "u0_err_max": float(np.abs(ug[:, :P.nu] - ur_[:, :P.nu]).max())}), flush=True)


def kernel_times(args):
    """Profiling driver: an FP32 solver of --batch instances of the benchmark's problem with a
    random iterate (N(0, 0.25) entries), instance tiles 1 per CTA, and single launches of the
    named round kernels (one untimed, then --kernel-reps timed with CUDA events on the solver's
    stream).  Prints kernel, ms per launch and algorithmic GB/s."""
    import torch
    import spock_gb300 as sg
    sg.build()
    B = args.batch
    path, _ = workload(args.seed, 1)
    t = sg.ScenarioTree(path)
    d = sg.ProblemData(t)
    c = sg.CacheBuilder(t, d).tol(TOL).andersonBuffer(ANDERSON).precision(32).batch(B).build()
    c.setTuning(1, 1, 1)
    g = torch.Generator(device="cuda").manual_seed(args.seed)
    z = (0.5 * torch.randn(c.sizeIterate(), B, device="cuda", generator=g)).contiguous()
    c.setIterateDevice(z.data_ptr(), 32)
    torch.cuda.synchronize()
    for k in args.kernels.split(","):
        ms, by = c.kernelTime(k, args.kernel_reps)
        print(json.dumps({"kernel": k, "batch": B, "ms": ms, "algorithmic_bytes": by,
                          "gbs": by / ms / 1e6 if by else None}), flush=True)


def gemm_times(args):
    """Profiling driver: spock_gemm_bf16 at the warm start's reconstruction shape (M = 138,760
    iterate entries, N = 1,024 instances, K = 384: BF16 hi/lo segments of 128 basis columns) and
    at an MLP shape (1,024 x 1,024, K = 2,048), three launches each, CUDA events."""
    import ctypes
    import torch
    import spock_gb300 as sg
    sg.build()
    vp = ctypes.c_void_p
    for (M, N, K) in [(138760, 1024, 384), (1024, 1024, 2048)]:
        A = torch.randn(M, K, device="cuda").to(torch.bfloat16)
        Bm = torch.randn(N, K, device="cuda").to(torch.bfloat16)
        D = torch.empty(M, N, device="cuda")
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            rc = sg.lib().spock_gemm_bf16(vp(A.data_ptr()), vp(Bm.data_ptr()), M, N, K, 1.0, None, None, 0,
                                          vp(D.data_ptr()), None, N, 0)
            e1.record()
            torch.cuda.synchronize()
            if rc:
                raise RuntimeError(sg.lib().spock_last_error().decode())
            ms = e0.elapsed_time(e1)
            print(json.dumps({"M": M, "N": N, "K": K, "ms": ms, "tflops": 2 * M * N * K / ms / 1e9,
                              "gbs_moved": (M * K * 2 + N * K * 2 + M * N * 4) / ms / 1e6}), flush=True)


def study_mixed(args):
    """Config 4's mixed batch: 256 problems, each from its own seed, nx ~ U{8..96}, nu = nx/2,
    Markov chains of 2-4 states, horizons 5-15, stopping stage 2-4, costs x 1e-3, one initial
    state each, FP32 SPOCK to tol(1e-4) with Anderson memory 5.  Timed: the group solve (every
    round one CUDA graph over all running solvers, spock_solve_group) and the same solves one
    after another.  Problems are written by a process pool before the GPU is touched."""
    from spock_gb300 import configs
    t0 = time.perf_counter()
    problems = configs.config4_mixed(PROBLEM_DIR, seed=args.seed, count=256, workers=os.cpu_count() or 1)
    print(json.dumps({"study": "mixed", "phase": "problems written", "seconds": round(time.perf_counter() - t0, 1)}),
          flush=True)
    import spock_gb300 as sg
    sg.build()
    caches, x0s, dims = [], [], []
    for path, x0 in problems:
        t = sg.ScenarioTree(path)
        d = sg.ProblemData(t)
        caches.append(sg.CacheBuilder(t, d).tol(TOL).andersonBuffer(ANDERSON).maxIters(args.max_iters).precision(32)
                      .batch(1).build())
        x0s.append(x0[None, :])
        dims.append((t.numStates(), t.numNodes()))
    sg.solve_group(caches, x0s)  # warm-up: each solver captures its round graph
    t0 = time.perf_counter()
    sts = sg.solve_group(caches, x0s)
    t_group = time.perf_counter() - t0
    it_group = np.array([c.solveIter() for c in caches])
    nx = np.array([q[0] for q in dims])
    nodes = np.array([q[1] for q in dims])
    base = {"study": "mixed", "problems": len(caches), "precision": "fp32", "tol": TOL,
            "nx_range": [int(nx.min()), int(nx.max())], "nodes_range": [int(nodes.min()), int(nodes.max())]}
    print(json.dumps(dict(base, method="group (one CUDA graph per round)", solves_per_s=len(caches) / t_group,
                          seconds=t_group, converged=int(sum(int(s[0] == 0) for s in sts)),
                          iters_mean=float(it_group.mean()), iters_max=int(it_group.max()))), flush=True)
    t0 = time.perf_counter()
    st_seq = [c.runSpock(x[0]) for c, x in zip(caches, x0s)]
    t_seq = time.perf_counter() - t0
    it_seq = np.array([c.solveIter() for c in caches])
    print(json.dumps(dict(base, method="one after another", solves_per_s=len(caches) / t_seq, seconds=t_seq,
                          converged=int(sum(s == 0 for s in st_seq)), iters_mean=float(it_seq.mean()),
                          iters_max=int(it_seq.max()), same_iterations=bool((it_seq == it_group).all()))), flush=True)


def study_finish(args):
    """The FP64 finish (spock_set_fp64_finish) on the benchmark's workload: from the same warm-up
    state, the K timed re-solve steps are run once per threshold in --finish-rounds (0: FP32
    throughout).  Per threshold: device-timed solves/s, rounds per step, outer iterations, and the
    largest relative difference of the optimal costs s_0 from the FP32-throughout run."""
    import torch
    import spock_gb300 as sg
    torch.cuda.set_device(0)
    sg.build()
    B = args.batch
    path, x0s = workload(args.seed, B)
    tree = sg.ScenarioTree(path)
    data = sg.ProblemData(tree)
    make = lambda: (sg.CacheBuilder(tree, data).tol(TOL).andersonBuffer(ANDERSON).maxIters(args.max_iters)
                    .precision(32).batch(B).build())
    cache, snap = make(), make()
    traj = trajectory(x0s, args.warmup + args.steps, args.seed)
    x_dev = [torch.tensor(x.T.copy(), dtype=torch.float32, device="cuda").contiguous() for x in traj]
    cache.runSpockBatch(x0s)
    for k in range(args.warmup):
        cache.resolveDevice(x_dev[k].data_ptr())
    snap.copyIterateFrom(cache)
    oS = tree.numNonleafNodes() * (tree.numInputs() + 2 * tree.numEvents() + 1) + tree.numNodes() * (
        tree.numStates() + 2) - tree.numNodes()
    base = None
    for R in [int(v) for v in args.finish_rounds.split(",")]:
        cache.copyIterateFrom(snap)
        cache.fp64Finish(R)
        if R > 0:  # the FP64 solver is made on first use: once, outside the timed steps
            cache.resolveDevice(x_dev[args.warmup].data_ptr())
            cache.copyIterateFrom(snap)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        conv, its, rounds = 0, [], 0
        for k in range(args.steps):
            st = cache.resolveDevice(x_dev[args.warmup + k].data_ptr())
            conv += int((st == 0).sum())
            its.append(cache.countersAll()[:, 6].copy())
            rounds += cache.runStats()[0]
        e1.record()
        torch.cuda.synchronize()
        sec = e0.elapsed_time(e1) / 1e3
        cost = cache.solutions()[:, oS]
        if base is None:
            base = cost
        its = np.concatenate(its)
        print(json.dumps({"study": "finish", "fp64_finish_rounds": R, "solves_per_s": B * args.steps / sec,
                          "converged": conv, "instances": B * args.steps, "rounds_per_step": rounds / args.steps,
                          "outer_iterations": {"mean": float(its.mean()), "max": int(its.max())},
                          "cost_rel_diff_vs_fp32_max": float(np.max(np.abs(cost - base) / np.abs(base)))}),
              flush=True)


def main():
    args = parse()
    if args.kernels:
        kernel_times(args)
        return
    if args.gemm:
        gemm_times(args)
        return
    if args.study == "mixed":
        study_mixed(args)
        return
    if args.study == "warmstart":
        study_warmstart(args)
        return
    if args.study == "precision":
        study_precision(args)
        return
    if args.study == "finish":
        study_finish(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
