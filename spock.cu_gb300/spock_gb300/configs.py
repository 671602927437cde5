"""Seeded synthetic RAOCP workloads (the five benchmark configurations).

Each builder writes a problem folder (data.json + .bt) with `factory` and returns
(path, x0) where x0 is a (count, nx) array of initial states drawn from the same seed.
Sizes:
  config1: 3-state Markov chain, N=4, tau=2 -> 31 nodes; nx=3, nu=2; quadratic costs;
           box |x|<=5, |u|<=2; AVaR(0.9); x0 ~ U[-1,1]^3; eps=1e-3, Anderson memory 3.
  config2: 3-state Markov chain, N=10, tau=4 -> 607 nodes; nx=50, nu=20; A_w ~ N(0,1/nx)
           rescaled to spectral radius 1.05, B_w ~ N(0,1); quadratic-plus-linear costs
           Q=diag U[1,10], R=diag U[0.1,1], q, r ~ N(0,1); box |x|<=3, |u|<=1; AVaR(0.95);
           x0 ~ U[-1,1]^50; eps=1e-4, Anderson memory 5.  `cost_scale` multiplies every cost
           term (Factory.with_cost_scaling); the benchmark uses 1e-3, because at the literal
           scale (cost-to-go near 800) SPOCK stalls near a residual of 1e-2.
  config3: i.i.d. process with 5 equiprobable events, N=8, tau=3 -> 781 nodes; nx=100, nu=40;
           dynamics generated as config2; quadratic costs; box |x|<=3 and the input ball
           ||u||_2 <= 2 (RectangleInputBall); AVaR(0.9).
  config4 uniform: config2 with `count` initial states (one problem, a batch of instances).
  config4 mixed (config4_mixed): `count` problems, each from its own seed, built like config2
           with nx ~ U{8..96}, nu = nx // 2, a Markov chain of 2-4 states, N ~ U{5..15},
           tau ~ U{2..4} (tau < N), costs x `cost_scale`; one initial state each.
"""
import os

import numpy as np

from . import factory as F

SOLVER = {
    "config1": dict(tol=1e-3, anderson=3),
    "config2": dict(tol=1e-4, anderson=5),
    "config3": dict(tol=1e-4, anderson=5),
}


def _stable_dynamics(rng, nx, nu, events, radius=1.05):
    out = []
    for _ in range(events):
        A = rng.normal(0., 1. / np.sqrt(nx), size=(nx, nx))
        A *= radius / max(abs(np.linalg.eigvals(A)))
        out.append(F.Dynamics(A, rng.standard_normal((nx, nu))))
    return out


def config1(path, seed=0, count=1):
    rng = np.random.default_rng(seed)
    ne, nx, nu = 3, 3, 2
    P = rng.dirichlet(np.ones(ne), size=ne)
    tree = F.MarkovChain(P, np.ones(ne) / ne, horizon=4, stopping_stage=2).build()
    dyn = [F.Dynamics(np.eye(nx) + .1 * rng.standard_normal((nx, nx)), rng.standard_normal((nx, nu)))
           for _ in range(ne)]
    Q = np.diag(rng.uniform(1., 10., nx))
    R = np.diag(rng.uniform(.1, 1., nu))
    lb = np.concatenate((-5. * np.ones(nx), -2. * np.ones(nu)))
    (F.Factory(tree, nx, nu).with_dynamics_events(dyn)
     .with_cost_nonleaf(F.CostQuadratic(Q, R))
     .with_cost_leaf(F.CostQuadratic(Q, leaf=True))
     .with_constraint_nonleaf(F.Rectangle(lb, -lb))
     .with_constraint_leaf(F.Rectangle(-5. * np.ones(nx), 5. * np.ones(nx)))
     .with_risk(F.AVaR(.9))
     .generate_problem(path))
    return path, rng.uniform(-1., 1., size=(count, nx))


def config2(path, seed=0, count=1, nx=50, nu=20, horizon=10, stopping=4, states=3, cost_scale=1., offline="host"):
    rng = np.random.default_rng(seed)
    P = rng.dirichlet(np.ones(states), size=states)
    tree = F.MarkovChain(P, np.ones(states) / states, horizon=horizon, stopping_stage=stopping).build()
    dyn = _stable_dynamics(rng, nx, nu, states)
    costs = [F.CostQuadraticPlusLinear(np.diag(rng.uniform(1., 10., nx)), rng.standard_normal(nx),
                                       np.diag(rng.uniform(.1, 1., nu)), rng.standard_normal(nu))
             for _ in range(states)]
    leaf = F.CostQuadraticPlusLinear(np.diag(rng.uniform(1., 10., nx)), rng.standard_normal(nx), leaf=True)
    lb = np.concatenate((-3. * np.ones(nx), -1. * np.ones(nu)))
    (F.Factory(tree, nx, nu).with_dynamics_events(dyn)
     .with_cost_nonleaf_events(costs)
     .with_cost_leaf(leaf)
     .with_constraint_nonleaf(F.Rectangle(lb, -lb))
     .with_constraint_leaf(F.Rectangle(-3. * np.ones(nx), 3. * np.ones(nx)))
     .with_risk(F.AVaR(.95))
     .with_cost_scaling(cost_scale)
     .generate_problem(path, offline=offline))
    return path, rng.uniform(-1., 1., size=(count, nx))


def config3(path, seed=0, count=1, nx=100, nu=40, horizon=8, stopping=3, events=5, radius=2., ball=True, cost_scale=1.,
            offline="host"):
    """Box |x| <= 3 on the states and the input ball ||u||_2 <= 2 (RectangleInputBall); the ball
    needs equal input scales, so this problem is not preconditioned.  With ball=False the input
    constraint is the box |u_i| <= radius instead (Rectangle, preconditioned): the variant the
    reference's constraint types can express.  `cost_scale` multiplies every cost term, as in
    config2.  offline="gpu" computes the offline cache on the GPU (Factory.generate_problem)."""
    rng = np.random.default_rng(seed)
    tree = F.IidProcess(np.ones(events) / events, horizon=horizon, stopping_stage=stopping).build()
    dyn = _stable_dynamics(rng, nx, nu, events)
    costs = [F.CostQuadratic(np.diag(rng.uniform(1., 10., nx)), np.diag(rng.uniform(.1, 1., nu)))
             for _ in range(events)]
    leaf = F.CostQuadratic(np.diag(rng.uniform(1., 10., nx)), leaf=True)
    (F.Factory(tree, nx, nu).with_dynamics_events(dyn)
     .with_cost_nonleaf_events(costs)
     .with_cost_leaf(leaf)
     .with_constraint_nonleaf(F.RectangleInputBall(-3. * np.ones(nx), 3. * np.ones(nx), nu, radius) if ball else
                              F.Rectangle(np.concatenate((-3. * np.ones(nx), -radius * np.ones(nu))),
                                          np.concatenate((3. * np.ones(nx), radius * np.ones(nu)))))
     .with_constraint_leaf(F.Rectangle(-3. * np.ones(nx), 3. * np.ones(nx)))
     .with_risk(F.AVaR(.9))
     .with_preconditioning(not ball)
     .with_cost_scaling(cost_scale)
     .generate_problem(path, offline=offline))
    return path, rng.uniform(-1., 1., size=(count, nx))


def _mixed_spec(root, seed, k, nx_range, states_range, horizon_range, stopping_range):
    rng = np.random.default_rng([seed, k])
    nx = int(rng.integers(nx_range[0], nx_range[1] + 1))
    states = int(rng.integers(states_range[0], states_range[1] + 1))
    horizon = int(rng.integers(horizon_range[0], horizon_range[1] + 1))
    stopping = int(min(rng.integers(stopping_range[0], stopping_range[1] + 1), horizon - 1))
    sub = int(rng.integers(0, 2 ** 31))
    path = os.path.join(root, f"config4_mixed_s{seed}", f"p{k:04d}", "")
    return path, dict(seed=sub, nx=nx, nu=max(1, nx // 2), horizon=horizon, stopping=stopping, states=states), \
        rng.uniform(-1., 1., size=nx)


def _mixed_write(job):
    path, kw, cost_scale = job
    if not os.path.exists(os.path.join(path, "data.json")):
        config2(path, cost_scale=cost_scale, **kw)
    return path


def config4_mixed(root, seed=0, count=256, nx_range=(8, 96), states_range=(2, 4), horizon_range=(5, 15),
                  stopping_range=(2, 4), cost_scale=1e-3, workers=1):
    """Write `count` problems under root/config4_mixed_s{seed}/p{k}/ (each kept if already there);
    returns [(path, x0)] with one initial state (nx,) per problem.  The ranges are inclusive.
    With workers > 1 the problems are written by a pool of processes (started by spawn)."""
    import json
    specs = [_mixed_spec(root, seed, k, nx_range, states_range, horizon_range, stopping_range) for k in range(count)]
    jobs = [(path, kw, cost_scale) for path, kw, _ in specs]
    if workers > 1:
        import multiprocessing as mp
        for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):  # one BLAS thread a worker
            os.environ.setdefault(var, "1")
        with mp.get_context("spawn").Pool(workers) as pool:
            pool.map(_mixed_write, jobs)
    else:
        for j in jobs:
            _mixed_write(j)
    out = []
    for path, kw, x0 in specs:
        assert json.load(open(os.path.join(path, "data.json")))["numStates"] == kw["nx"]
        out.append((path, x0))
    return out


BUILDERS = {"config1": config1, "config2": config2, "config3": config3}


def cached(name, root, seed=0, count=1, **kw):
    """Build a configuration once under `root/name_s{seed}` and reuse it afterwards."""
    path = os.path.join(root, f"{name}_s{seed}" + "".join(f"_{k}{v}" for k, v in sorted(kw.items())), "")
    if not os.path.exists(os.path.join(path, "data.json")):
        BUILDERS[name](path, seed=seed, count=1, **kw)
    rng = np.random.default_rng(seed + 7919)
    import json
    nx = json.load(open(os.path.join(path, "data.json")))["numStates"]
    return path, rng.uniform(-1., 1., size=(count, nx))
