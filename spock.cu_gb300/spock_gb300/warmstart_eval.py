"""Evaluate the learned warm start on the benchmark problem family (reduced config 5).

    python -m spock_gb300.warmstart_eval [--train 2048] [--train-tol 1e-4] [--test 1024] [--epochs 40]

(run from spock.cu_gb300/, or with it on sys.path).  Training data: cold FP32 batch solves of
`--train` initial states x0 ~ U[-1, 1]^50 of config 2 with costs x 1e-3 (the benchmark problem)
at tol(--train-tol); config 5 names 200k solves at 1e-5, which this problem's iteration does not
reach in reasonable time (the FP64 oracle converges for 2 of 8 cold starts within 4,000 outer
iterations; FP32 also suffers from the float accumulation of its forward dynamics rollout).
Model: PCA(128) of the solutions + MLP 50 -> 1024 -> 1024 -> 128 (GELU, BF16
weights, FP32 accumulation), trained with the library's kernels.  Evaluation: `--test` held-out
x0 in one batch, solved to tol(1e-4) in FP32 (i) cold, (ii) cold to the absolute tolerance only
(the tolerance a warm start meets), (iii) from the MLP's predicted iterate and (iv) from the
solution of the nearest training x0; prints one JSON line per method with solves/s,
mean / max outer iterations and the error of u_0 against the cold solve.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def main():
    import torch
    import spock_gb300 as sg
    from spock_gb300 import configs
    from spock_gb300.warmstart import PcaMlpWarmStart
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=2048)
    ap.add_argument("--train-tol", type=float, default=1e-4)
    ap.add_argument("--test", type=int, default=1024)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--dir", default=os.environ.get("SPOCK_BENCH_DIR", "/tmp/spock_bench"))
    args = ap.parse_args()
    sg.build()
    B = args.test
    path, _ = configs.cached("config2", args.dir, seed=0, count=1, cost_scale=1e-3)
    rng = np.random.default_rng(2026)
    xtr = rng.uniform(-1., 1., (args.train, 50))
    xte = rng.uniform(-1., 1., (B, 50))
    t = sg.ScenarioTree(path)
    d = sg.ProblemData(t)

    def cache(tol):
        return (sg.CacheBuilder(t, d).tol(tol).andersonBuffer(5).maxIters(20000).precision(32).batch(B).build())

    # training data
    t0 = time.time()
    ctr = cache(args.train_tol)
    zs = []
    for s in range(0, args.train, B):
        ctr.runSpockBatch(xtr[s:s + B])
        zs.append(torch.tensor(ctr.solutions(), dtype=torch.float32, device="cuda"))
    zs = torch.cat(zs)
    print(json.dumps({"phase": "data", "solves": args.train, "seconds": round(time.time() - t0, 1)}), flush=True)
    t0 = time.time()
    ws = PcaMlpWarmStart(k=128, hidden=1024, seed=0)
    losses = ws.fit(xtr, zs, epochs=args.epochs, batch=min(1024, args.train), lr=1e-3)
    print(json.dumps({"phase": "fit", "seconds": round(time.time() - t0, 1), "loss_first": losses[0],
                      "loss_last": losses[-1], "pca_explained": ws.explained}), flush=True)

    def run(name, prepare, absolute=False):
        c = cache(1e-4) if not absolute else (sg.CacheBuilder(t, d).toleranceAbsolute(1e-4).toleranceRelative(0.)
                                              .andersonBuffer(5).maxIters(20000).precision(32).batch(B).build())
        prepare(c)
        torch.cuda.synchronize()
        t1 = time.time()
        st = c.resolveBatch(xte) if not name.startswith("cold") else c.runSpockBatch(xte)
        el = time.time() - t1
        it = c.solveIters()
        return c, {"method": name, "solves_per_s": B / el, "seconds": round(el, 2), "converged": int((st == 0).sum()),
                   "iters_mean": float(it.mean()), "iters_max": int(it.max())}

    cold, rec = run("cold", lambda c: None)
    u_cold = cold.firstInputs()
    print(json.dumps(rec), flush=True)
    # a warm start captures a small initial error, so its stopping tolerance is the absolute one;
    # the same absolute tolerance from a cold start is the comparison at equal accuracy
    _, rec = run("cold_absolute_tol", lambda c: None, absolute=True)
    print(json.dumps(rec), flush=True)
    warm, rec = run("learned", lambda c: ws.warm_start(c, xte))
    rec["u0_err_vs_cold"] = float(np.abs(warm.firstInputs() - u_cold).max())
    print(json.dumps(rec), flush=True)
    nearest = np.argmin(((xte[:, None, :] - xtr[None, :, :]) ** 2).sum(-1), axis=1)

    def nearest_prep(c):
        z = zs[torch.tensor(nearest, device="cuda")].T.contiguous()
        c.setIterateDevice(z.data_ptr(), 32)

    near, rec = run("nearest_training_solution", nearest_prep)
    rec["u0_err_vs_cold"] = float(np.abs(near.firstInputs() - u_cold).max())
    print(json.dumps(rec), flush=True)


if __name__ == "__main__":
    main()
