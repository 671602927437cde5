"""Parity of the CUDA path (through the C ABI) with the FP64 CPU oracle.

Tolerances: FP64 kernels must agree with the oracle to 1e-10 relative (same arithmetic up to
summation order); FP32 kernels to 2e-5 relative to the vector's scale (single precision).
Solves are compared on the solution they return: FP64 to 1e-6, FP32 to 1e-3 relative.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden

import spock_gb300 as sg

pytestmark = pytest.mark.gpu

CASES = ["reftest", "cfg1", "qpl"]
GOLDEN_CASES_ALL = ["reftest", "cfg1", "qpl", "affpoly"]


@pytest.fixture(scope="module", autouse=True)
def built():
    sg.build()


def make(path, precision=64, batch=1, tol=1e-3, max_iters=0, anderson=3):
    t = sg.ScenarioTree(path)
    d = sg.ProblemData(t)
    c = (sg.CacheBuilder(t, d).tol(tol).maxIters(max_iters).andersonBuffer(anderson)
         .precision(precision).batch(batch).build())
    return t, d, c


def x0_of(case, nx):
    return golden(case, "initialState_d.bt") if case != "reftest" else np.full(nx, 1.1)


def rel(a, b):
    return np.abs(a - b).max() / max(1., np.abs(b).max())


BATCHES = [1, 32]  # 1: per-row kernels (kernels.cuh); 32: batched kernels (kernels_batch.cuh)


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("precision,tol", [(64, 1e-12), (32, 2e-5)])
@pytest.mark.parametrize("batch", BATCHES)
def test_operators(oracle_lib, case, precision, tol, batch):
    path = os.path.join(GOLDEN, case)
    t, d, c = make(path, precision, batch=batch)
    P = oracle_lib.Problem(path)
    prim = golden(case, "test_primBeforeOp_d.bt")
    dual = golden(case, "test_dualAfterOpBeforeAdj_d.bt")
    assert rel(c.op(prim), dual) < tol
    assert rel(c.adj(dual), golden(case, "test_primAfterAdj_d.bt")) < tol
    rng = np.random.default_rng(5)
    z = rng.standard_normal(c.sizeIterate())
    assert rel(c.applyM(z), np.concatenate((z[:P.size_prim] - P.step * P.adj(z[P.size_prim:]),
                                             z[P.size_prim:] - P.step * P.op(z[:P.size_prim])))) < tol
    v = golden(case, "test_dotVector_d.bt")
    ref = golden(case, "test_dotResult_d.bt")[0]
    assert abs(c.dotM(v, v) - ref) <= (1e-9 if precision == 64 else 1e-5) * abs(ref)


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("precision,tol", [(64, 1e-10), (32, 1e-4)])
@pytest.mark.parametrize("batch", BATCHES)
def test_cp_step(oracle_lib, case, precision, tol, batch):
    """One Chambolle-Pock step T(z) (cache.cuh:795-801) from random iterates."""
    path = os.path.join(GOLDEN, case)
    t, d, c = make(path, precision, batch=batch)
    P = oracle_lib.Problem(path)
    x0 = x0_of(case, P.nx)
    rng = np.random.default_rng(11)
    for _ in range(3):
        z = 3 * rng.standard_normal(P.size)
        assert rel(c.cpStep(x0, z), P.cp_step(x0 * P.scaling[:P.nx], z)) < tol


@pytest.mark.parametrize("case", CASES)
def test_cp_solve_fp64(oracle_lib, case):
    """runCp: deterministic, so the GPU and the oracle take the same iterations."""
    path = os.path.join(GOLDEN, case)
    t, d, c = make(path, 64, tol=1e-3, max_iters=3000)
    P = oracle_lib.Problem(path)
    x0 = x0_of(case, P.nx)
    st = c.runCp(x0)
    z, s = P.run(x0, oracle_lib.options(tol=1e-3, max_iters=3000), "cp")
    assert st == s.status
    assert c.solveIter() == s.iters
    assert rel(c.solution(), z) < 1e-8


@pytest.mark.parametrize("case", CASES)
def test_spock_solve_fp64(oracle_lib, case):
    """runSpock to tol 1e-3 (testCache.cu:294-308) in FP64: converged, same solution as the
    oracle's SuperMann run."""
    path = os.path.join(GOLDEN, case)
    t, d, c = make(path, 64, tol=1e-3, max_iters=3000)
    P = oracle_lib.Problem(path)
    x0 = x0_of(case, P.nx)
    assert c.runSpock(x0) == 0
    z, s = P.run(x0, oracle_lib.options(tol=1e-3, max_iters=3000), "spock")
    assert s.status == 0
    assert abs(c.solveIter() - s.iters) <= 50
    # Both stop at the same tolerance, but the GPU's Anderson step solves the Gram normal
    # equations where the oracle uses Householder QR, so the two trajectories end at different
    # points of the tolerance band.  The GPU's solution must pass the reference's termination
    # test (cache.cuh:909-961) as the oracle evaluates it.
    x0s = x0 * P.scaling[:P.nx]
    zg = c.solution()
    r = zg - P.cp_step(x0s, zg)
    sp = P.size_prim
    mr = np.concatenate((r[:sp] - P.step * P.adj(r[sp:]), r[sp:] - P.step * P.op(r[:sp])))
    assert np.abs(mr).max() / P.step <= 3 * s.tol


def test_tight_solve_matches_oracle(oracle_lib):
    """Reference test problem solved to 1e-10 (both converge): first-stage input and optimal
    value s_0 agree to 1e-8 (FP64) and the FP32 path agrees to 1e-4."""
    path = os.path.join(GOLDEN, "reftest")
    P = oracle_lib.Problem(path)
    x0 = np.full(P.nx, 1.1)
    z, s = P.run(x0, oracle_lib.options(tol=1e-10, max_iters=20000), "spock")
    assert s.status == 0
    s0 = P.size_prim - P.n
    for prec, tol, eps in [(64, 1e-8, 1e-10), (32, 1e-4, 1e-6)]:
        t, d, c = make(path, prec, tol=eps, max_iters=20000)
        st = c.runSpock(x0)
        assert st == 0 or prec == 32
        zg = c.solution()
        assert abs(zg[s0] - z[s0]) <= tol * abs(z[s0])
        assert np.abs(c.inputs()[:P.nu] - P.states_inputs(z)[1][:P.nu]).max() <= tol * 10


def test_batched_fp32_matches_single(oracle_lib):
    """A batch of 24 cfg1 instances with distinct initial states: every instance converges and
    its first input matches the oracle's FP64 single solve."""
    path = os.path.join(GOLDEN, "cfg1")
    P = oracle_lib.Problem(path)
    rng = np.random.default_rng(3)
    x0s = rng.uniform(-1, 1, (24, P.nx))
    t, d, c = make(path, 32, batch=24, tol=1e-3, max_iters=3000)
    st = c.runSpockBatch(x0s)
    assert (st == 0).all()
    u0 = c.firstInputs()
    for b in range(24):
        z, s = P.run(x0s[b], oracle_lib.options(tol=1e-3, max_iters=3000), "spock")
        u_ref = P.states_inputs(z)[1][:P.nu]
        assert np.abs(u0[b] - u_ref).max() <= 2e-2 * max(1., np.abs(u_ref).max()), b


@pytest.mark.parametrize("case", ["cfg1", "qpl"])
def test_batched_kernels_solve(oracle_lib, case):
    """64 instances through the batched kernels (FP32): all converge and their first inputs
    match the oracle's FP64 solves.  (The reference test problem's terminal box |x| <= 0.1 is
    infeasible for many random initial states, so it is not used here.)"""
    path = os.path.join(GOLDEN, case)
    P = oracle_lib.Problem(path)
    rng = np.random.default_rng(8)
    x0s = rng.uniform(-1, 1, (64, P.nx))
    t, d, c = make(path, 32, batch=64, tol=1e-3, max_iters=3000)
    st = c.runSpockBatch(x0s)
    assert (st == 0).all()
    u0 = c.firstInputs()
    for b in range(0, 64, 9):
        z, s = P.run(x0s[b], oracle_lib.options(tol=1e-3, max_iters=3000), "spock")
        u_ref = P.states_inputs(z)[1][:P.nu]
        assert np.abs(u0[b] - u_ref).max() <= 2e-2 * max(1., np.abs(u_ref).max()), b


def test_batch_rows_reused_cyclically(oracle_lib):
    path = os.path.join(GOLDEN, "cfg1")
    t, d, c = make(path, 64, batch=4, tol=1e-3, max_iters=1000)
    x0 = golden("cfg1", "initialState_d.bt")
    st = c.runSpockBatch(x0[None, :])
    assert (st == 0).all()
    u0 = c.firstInputs()
    assert np.allclose(u0, u0[0][None, :], atol=1e-12)


def test_warm_start_from_solution(oracle_lib):
    """A warm start at the solution (the previousSolution path, cache.cuh:611-632): the first
    error check captures the absolute tolerance (the warm start's error is small), which the
    re-solve then reaches.  The oracle takes the same path from its own solution; the iteration
    counts agree to two error-check periods (SuperMann paths diverge with rounding)."""
    path = os.path.join(GOLDEN, "cfg1")
    t, d, c = make(path, 64, tol=1e-3, max_iters=3000)
    x0 = golden("cfg1", "initialState_d.bt")
    assert c.runSpock(x0) == 0
    z = c.solution()
    assert c.runSpock(x0, prev=z) == 0
    P = oracle_lib.Problem(path)
    opts = oracle_lib.options(tol=1e-3, max_iters=3000)
    z_ref, st = P.run(x0, opts)
    _, st_warm = P.run(x0, opts, z=z_ref)
    assert st_warm.status == 0
    assert abs(c.solveIter() - st_warm.iters) <= 50, (c.solveIter(), st_warm.iters)


@pytest.mark.parametrize("batch", [1, 32])
@pytest.mark.parametrize("precision,tol", [(64, 1e-12), (32, 2e-5)])
def test_linear_costs_polyhedra_affine(oracle_lib, batch, precision, tol):
    """Affine dynamics, linear costs and polyhedral constraints (the reference factory's affpoly
    fixture): L and L* against the reference's own vectors, one CP step from random iterates
    against the oracle, and 200 plain CP iterations taking the oracle's path (FP64)."""
    case = "affpoly"
    path = os.path.join(GOLDEN, case)
    t, d, c = make(path, precision, batch=batch)
    P = oracle_lib.Problem(path)
    prim = golden(case, "test_primBeforeOp_d.bt")
    dual = golden(case, "test_dualAfterOpBeforeAdj_d.bt")
    assert rel(c.op(prim), dual) < tol
    assert rel(c.adj(dual), golden(case, "test_primAfterAdj_d.bt")) < tol
    rng = np.random.default_rng(31)
    x0 = rng.uniform(-1, 1, P.nx)
    for _ in range(3):
        z = 3 * rng.standard_normal(P.size)
        assert rel(c.cpStep(x0, z), P.cp_step(x0, z)) < (1e-10 if precision == 64 else 1e-4)
    if precision == 64:
        t2, d2, c2 = make(path, 64, batch=batch, tol=1e-12, max_iters=200)
        c2.runCp(x0)
        z, s = P.run(x0, oracle_lib.options(tol=1e-12, max_iters=200), "cp")
        assert rel(c2.solution(), z) < 1e-8


@pytest.mark.parametrize("batch", BATCHES)
def test_full_size_operator_parity(oracle_lib, tmp_problems, batch):
    """Config-2 sized problem (607 nodes, nx=50, nu=20): FP64 L, L*, T and M against the
    oracle, and the adjoint identity in FP32."""
    from spock_gb300 import configs
    path, x0 = configs.cached("config2", tmp_problems, seed=0, count=1)
    P = oracle_lib.Problem(path)
    t, d, c = make(path, 64, batch=batch)
    rng = np.random.default_rng(2)
    p = rng.standard_normal(P.size_prim)
    q = rng.standard_normal(P.size_dual)
    assert rel(c.op(p), P.op(p)) < 1e-12
    assert rel(c.adj(q), P.adj(q)) < 1e-12
    z = rng.standard_normal(P.size)
    assert rel(c.cpStep(x0[0], z), P.cp_step(x0[0] * P.scaling[:P.nx], z)) < 1e-10
    t32, d32, c32 = make(path, 32, batch=batch)
    lhs, rhs = q @ c32.op(p), c32.adj(q) @ p
    assert abs(lhs - rhs) <= 1e-4 * max(abs(lhs), 1.)


@pytest.mark.parametrize("batch", BATCHES)
def test_full_size_dynamics_feasible(oracle_lib, tmp_problems, batch):
    """After one FP32 CP step on a config-2 problem the candidate (x, u) satisfies the
    dynamics x_j = A_j x_anc(j) + B_j u_anc(j) and x_0 = x0 (the projection's defining
    property, dynamics.cuh:74-174)."""
    from spock_gb300 import configs
    from spock_gb300.factory import read_bt
    path, x0 = configs.cached("config2", tmp_problems, seed=0, count=1)
    P = oracle_lib.Problem(path)
    t, d, c = make(path, 32, batch=batch)
    z = np.random.default_rng(4).standard_normal(P.size)
    cand = c.cpStep(x0[0], z)
    nx, nu, n, nnl = P.nx, P.nu, P.n, P.nnl
    u = cand[:nu * nnl].reshape(nnl, nu)
    x = cand[nu * nnl:nu * nnl + nx * n].reshape(n, nx)
    AB = read_bt(path + "dynamics_AB_d.bt")
    anc = read_bt(path + "ancestors_u.bt").ravel().astype(np.int64)
    assert np.allclose(x[0], x0[0] * P.scaling[:nx], atol=1e-6)
    pred = np.einsum("rcn,nc->nr", AB[:, :, 1:], np.concatenate((x[anc[1:]], u[anc[1:]]), axis=1))
    assert np.abs(pred - x[1:]).max() <= 1e-4 * max(1., np.abs(x).max())


def test_resolve_from_previous_solution(oracle_lib):
    """spock_resolve: 32 instances of the reference's test problem re-solved warm from their
    previous solutions after a small move of x0 (the previousSolution path, cache.cuh:611-632,
    kept on the device) converge, and their first inputs agree with cold solves of the same
    states."""
    path = os.path.join(GOLDEN, "reftest")
    P = oracle_lib.Problem(path)
    x0s = np.full((32, P.nx), 1.1) + np.linspace(-.05, .05, 32)[:, None]
    t, d, c = make(path, 64, batch=32, tol=1e-8, max_iters=20000)
    assert (c.runSpockBatch(x0s) == 0).all()
    x1 = x0s + np.random.default_rng(21).uniform(-.01, .01, x0s.shape)
    assert (c.resolveBatch(x1) == 0).all()
    u_warm = c.firstInputs()
    t2, d2, c2 = make(path, 64, batch=32, tol=1e-8, max_iters=20000)
    assert (c2.runSpockBatch(x1) == 0).all()
    assert np.abs(u_warm - c2.firstInputs()).max() <= 1e-5 * max(1., np.abs(c2.firstInputs()).max())


def test_converged_instances_stay_put(oracle_lib):
    """Per-instance convergence masks: in a batch whose instances stop at very different
    iterations (the first tile starts at its own solution, the second cold), the early ones keep
    the solution they stopped at while the node kernels skip their tile."""
    path = os.path.join(GOLDEN, "reftest")
    P = oracle_lib.Problem(path)
    x0s = np.full((64, P.nx), 1.1) + np.linspace(-.05, .05, 64)[:, None]
    t, d, c = make(path, 64, batch=64, tol=1e-8, max_iters=20000)
    assert (c.runSpockBatch(x0s) == 0).all()
    z = c.solutions()
    warm = z.copy()
    warm[32:] = 0.
    assert (c.runSpockBatch(x0s, prev=warm) == 0).all()
    it = c.solveIters()
    assert it[:32].max() < it[32:].min()
    assert np.abs(c.solutions()[:32] - z[:32]).max() <= 1e-6 * max(1., np.abs(z).max())


@pytest.mark.parametrize("case", CASES)
def test_offline_dynamics_cache_on_gpu(case):
    """spock_offline_dynamics: the dynamics cache (problem.py:192-213) recomputed on the GPU in
    FP64 matches the reference factory's own files to 1e-10 relative."""
    t = sg.ScenarioTree(os.path.join(GOLDEN, case))
    out = t.offlineDynamics(replace=False)
    for name, key in [("P", "P"), ("K", "K"), ("lowCholesky", "lowChol"), ("ABKTr", "ABKTr"), ("APB", "APB")]:
        ref = golden(case, f"dynamics_{name}_d.bt")
        assert np.abs(out[key] - ref).max() <= 1e-10 * max(1., np.abs(ref).max()), name


def test_fp64_polish_of_fp32_solve(oracle_lib):
    """FP32 batch solve to 1e-3, handed over on the device to an FP64 solver that polishes to
    1e-9 (spock_copy_iterate + spock_resolve): every instance converges and u_0 agrees with the
    oracle's FP64 solve at 1e-9 to 1e-6."""
    path = os.path.join(GOLDEN, "reftest")
    P = oracle_lib.Problem(path)
    x0s = np.full((32, P.nx), 1.1) + np.linspace(-.05, .05, 32)[:, None]
    t, d, c32 = make(path, 32, batch=32, tol=1e-3, max_iters=20000)
    assert (c32.runSpockBatch(x0s) == 0).all()
    t2, d2, c64 = make(path, 64, batch=32, tol=1e-9, max_iters=20000)
    assert (c64.polish(c32, x0s) == 0).all()
    u0 = c64.firstInputs()
    oS = P.size_prim - P.n  # the optimal cost: s at the root
    for b in (0, 31):
        z, s = P.run(x0s[b], oracle_lib.options(tol=1e-9, max_iters=20000), "spock")
        u_ref = P.states_inputs(z)[1][:P.nu]
        assert np.abs(u0[b] - u_ref).max() <= 1e-6 * max(1., np.abs(u_ref).max()), b
        assert abs(c64.solution(b)[oS] - z[oS]) <= 1e-6 * abs(z[oS]), b


@pytest.mark.parametrize("batch", [1, 32])
def test_input_ball_constraint(oracle_lib, tmp_problems, batch):
    """The input-ball constraint ||u||_2 <= r of config 3 on a small problem: the T step matches
    the oracle (FP64 1e-10, FP32 1e-4), and an FP64 SPOCK solve converges with the oracle's u_0
    and keeps every input inside the ball."""
    from spock_gb300 import configs
    path, x0 = configs.cached("config3", tmp_problems, seed=1, count=1, nx=4, nu=3, horizon=3, stopping=2,
                              events=2, radius=.5)
    P = oracle_lib.Problem(path)
    rng = np.random.default_rng(41)
    for prec, tol in [(64, 1e-10), (32, 1e-4)]:
        t, d, c = make(path, prec, batch=batch)
        for _ in range(3):
            z = 3 * rng.standard_normal(P.size)
            assert rel(c.cpStep(x0[0], z), P.cp_step(x0[0], z)) < tol
    t, d, c = make(path, 64, batch=batch, tol=1e-8, max_iters=20000)
    assert c.runSpock(x0[0]) == 0
    z, s = P.run(x0[0], oracle_lib.options(tol=1e-8, max_iters=20000), "spock")
    assert s.status == 0
    u_ref = P.states_inputs(z)[1]
    u = c.inputs()
    assert np.abs(u[:P.nu] - u_ref[:P.nu]).max() <= 1e-5 * max(1., np.abs(u_ref).max())
    assert np.linalg.norm(u.reshape(-1, P.nu), axis=1).max() <= .5 * (1 + 1e-4)


def test_instance_compaction(oracle_lib):
    """Instance compaction: in a batch of 128 where every fourth instance starts cold and the others
    at their solution, the cold ones -- spread over all four tiles -- are moved to the leading slots
    once the warm ones stop.  Every instance still converges to its own solution (u_0 against the
    oracle), and the warm ones keep theirs."""
    path = os.path.join(GOLDEN, "reftest")
    P = oracle_lib.Problem(path)
    x0s = np.full((128, P.nx), 1.1) + np.linspace(-.05, .05, 128)[:, None]
    t, d, c = make(path, 64, batch=128, tol=1e-8, max_iters=20000)
    assert (c.runSpockBatch(x0s) == 0).all()
    z = c.solutions()
    warm = z.copy()
    warm[::4] = 0.
    assert (c.runSpockBatch(x0s, prev=warm) == 0).all()
    assert c.compactions() >= 1
    u0 = c.firstInputs()
    for b in (0, 4, 124):
        zr, s = P.run(x0s[b], oracle_lib.options(tol=1e-8, max_iters=20000), "spock")
        u_ref = P.states_inputs(zr)[1][:P.nu]
        assert np.abs(u0[b] - u_ref).max() <= 1e-6 * max(1., np.abs(u_ref).max()), b
    keep = np.ones(128, bool)
    keep[::4] = False
    assert np.abs(c.solutions()[keep] - z[keep]).max() <= 1e-6 * max(1., np.abs(z).max())


def test_mixed_batch_solve_group(oracle_lib):
    """Mixed batch (instances of different trees and dimensions): three problems solved at once by
    spock_solve_group, one host thread and stream each, give exactly the solutions and iteration
    counts of the same solves run one after another."""
    specs = [("reftest", 64, 1, np.full((1, 3), 1.1)), ("cfg1", 32, 40, None), ("qpl", 64, 8, None)]
    rng = np.random.default_rng(51)
    caches, alone, x0s = [], [], []
    for case, prec, batch, x0 in specs:
        path = os.path.join(GOLDEN, case)
        P = oracle_lib.Problem(path)
        x = x0 if x0 is not None else rng.uniform(-1, 1, (batch, P.nx))
        x0s.append(x)
        t, d, c = make(path, prec, batch=batch, tol=1e-3, max_iters=3000)
        caches.append(c)
        t2, d2, c2 = make(path, prec, batch=batch, tol=1e-3, max_iters=3000)
        c2.runSpockBatch(x)
        alone.append(c2)
    sts = sg.solve_group(caches, x0s)
    for c, c2, st in zip(caches, alone, sts):
        assert (st == c2.statuses()).all() and (st == 0).all()
        assert (c.solveIters() == c2.solveIters()).all()
        assert np.array_equal(c.solutions(), c2.solutions())


@pytest.mark.parametrize("case", GOLDEN_CASES_ALL)
def test_step_size_on_gpu(case):
    """spock_step_size: 0.99 / ||L|| from the power iteration on the GPU (FP64, the library's own L
    and L* kernels) matches the step size the reference factory wrote (ARPACK, problem.py:402-417)."""
    import json
    path = os.path.join(GOLDEN, case)
    ref = json.load(open(os.path.join(path, "data.json")))["stepSize"]
    t, d, c = make(path, 64)
    lam, step = c.stepSize(20000)
    assert abs(step - ref) <= 1e-6 * ref


@pytest.mark.parametrize("batch", BATCHES)
def test_polyhedron_with_identity(oracle_lib, tmp_path, batch):
    """[I; Gamma] constraints on nonleaf and leaf nodes (constraints.cuh:296-426), preconditioned:
    L, L* and the T step against the oracle (FP64 1e-10, FP32 1e-4), and an FP64 SPOCK solve
    with the oracle's u_0."""
    from test_factory import build_polyid
    path = str(tmp_path) + "/"
    build_polyid(path)
    P = oracle_lib.Problem(path)
    rng = np.random.default_rng(43)
    x0 = rng.uniform(-.5, .5, P.nx)
    p, q = rng.standard_normal(P.size_prim), rng.standard_normal(P.size_dual)
    for prec, tol in [(64, 1e-10), (32, 1e-4)]:
        t, d, c = make(path, prec, batch=batch)
        assert rel(c.op(p), P.op(p)) < tol
        assert rel(c.adj(q), P.adj(q)) < tol
        for _ in range(3):
            z = 3 * rng.standard_normal(P.size)
            assert rel(c.cpStep(x0, z), P.cp_step(x0 * P.scaling[:P.nx], z)) < tol
    t, d, c = make(path, 64, batch=batch, tol=1e-8, max_iters=20000)
    assert c.runSpock(x0) == 0
    z, s = P.run(x0, oracle_lib.options(tol=1e-8, max_iters=20000), "spock")
    assert s.status == 0
    u_ref = P.states_inputs(z)[1][:P.nu]
    assert np.abs(c.inputs()[:P.nu] - u_ref).max() <= 1e-5 * max(1., np.abs(u_ref).max())


@pytest.mark.parametrize("precision,tol,batch", [(64, 1e-10, 1), (32, 1e-4, 32)])
def test_get_dual(oracle_lib, precision, tol, batch):
    """Cache::getDual (cache.cuh:371-376): at the iterate z, the dual candidate for the primal
    half of T(z) is the dual half of T(z) (the oracle's CP step)."""
    path = os.path.join(GOLDEN, "cfg1")
    t, d, c = make(path, precision, batch=batch)
    P = oracle_lib.Problem(path)
    x0 = golden("cfg1", "initialState_d.bt")
    z = np.random.default_rng(12).standard_normal(P.size)
    c.cpStep(x0, z)  # leaves z as the solver's iterate
    ref = P.cp_step(x0 * P.scaling[:P.nx], z)
    assert rel(c.getDual(ref[:P.size_prim]), ref[P.size_prim:]) < tol
