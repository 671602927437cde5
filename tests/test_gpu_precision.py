"""Full-size parity of the larger problems and the FP32 path's accuracy against FP64.

* Config 3 (i.i.d. process with 5 events, N=8, stopping stage 3: 781 nodes; nx=100, nu=40): one
  CP step T(z) from random iterates through the batched kernels, FP64 and FP32, against the
  oracle; with the input ball ||u||_2 <= 2 (a constraint the reference has no class for) and
  with the input box the reference can express (src/constraints.cuh:70-74).
  FP64 with the input ball needs more shared memory than an SM has at this size, and is
  rejected with a message.
* The FP32 dynamics projection (dynamics.cuh:74-174) on config 2 against the FP64 projection:
  with the compensated forward rollout (and d from the FP64-derived inverse) its error is at
  most 0.75 of what plain float accumulation gives; the oracle's FP32 emulation measures the
  latter on float-rounded data (about 3.7e-7 relative; Dot2 in the emulation: 2.0e-7).
"""
import numpy as np
import pytest

from test_gpu_parity import make, rel

import spock_gb300 as sg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ball", [True, False])
@pytest.mark.parametrize("precision,tol", [(64, 1e-10), (32, 1e-4)])
def test_config3_full_size_step(oracle_lib, tmp_problems, ball, precision, tol):
    from spock_gb300 import configs
    path, x0 = configs.cached("config3", tmp_problems, seed=0, count=1, ball=ball)
    P = oracle_lib.Problem(path)
    assert (P.n, P.nx, P.nu) == (781, 100, 40)
    if precision == 64 and ball:
        with pytest.raises(ValueError, match="too large"):
            make(path, precision, batch=32)
        return
    t, d, c = make(path, precision, batch=32)
    rng = np.random.default_rng(5)
    for _ in range(2):
        z = rng.standard_normal(P.size)
        assert rel(c.cpStep(x0[0], z), P.cp_step(x0[0] * P.scaling[:P.nx], z)) < tol


def test_fp32_projection_error_against_fp64(oracle_lib, tmp_problems):
    from spock_gb300 import configs
    path, x0 = configs.cached("config2", tmp_problems, seed=0, count=1, cost_scale=1e-3)
    P0 = oracle_lib.Problem(path)
    rng = np.random.default_rng(0)
    x = rng.standard_normal(P0.nx * P0.n).astype(np.float32).astype(np.float64)
    u = rng.standard_normal(P0.nu * P0.nnl).astype(np.float32).astype(np.float64)
    x0s = (x0[0] * P0.scaling[:P0.nx]).astype(np.float32).astype(np.float64)
    D, A, V = oracle_lib.EMU_DATA, oracle_lib.EMU_ACC, oracle_lib.EMU_VEC
    ref = np.concatenate(P0.project_dynamics(x0s, x, u))
    try:
        oracle_lib.set_emulation(D | A | V)
        plain = np.concatenate(oracle_lib.Problem(path).project_dynamics(x0s, x, u))
    finally:
        oracle_lib.set_emulation(0)
    err_plain = np.abs(plain - ref).max() / np.abs(ref).max()
    # the GPU's projection: a T step from z = [u x 0 ...] with a zero dual part leaves (u, x)
    # equal to the projection of z's (u, x) (the L* term vanishes)
    t, d, c = make(path, 32, batch=32)
    z = np.zeros(P0.size)
    z[:P0.nu * P0.nnl] = u
    z[P0.nu * P0.nnl:P0.nu * P0.nnl + P0.nx * P0.n] = x
    cand = c.cpStep(x0[0], z)  # scaled and rounded to float by the solver, as x0s above
    gpu = np.concatenate((cand[P0.nu * P0.nnl:P0.nu * P0.nnl + P0.nx * P0.n], cand[:P0.nu * P0.nnl]))
    err_gpu = np.abs(gpu - ref).max() / np.abs(ref).max()
    print(f"FP32 projection error vs FP64: GPU {err_gpu:.3g}, emulated plain float {err_plain:.3g}")
    assert err_gpu < 0.75 * err_plain, (err_gpu, err_plain)


@pytest.mark.parametrize("batch", [1, 64])
def test_fp32_round_reductions_against_fp64(oracle_lib, tmp_problems, batch):
    """The round's reductions of an FP32 solver (k_reduce: blocks of 32 rows summed in float,
    running sums as float pairs, partials widened to FP64) on a config-2 sized residual
    (138,760 entries): r'Mr, max|Mr| and r'r against FP64 sums of the same float-rounded
    vectors, to 1e-6 relative."""
    from spock_gb300 import configs
    path, _ = configs.cached("config2", tmp_problems, seed=0, count=1, cost_scale=1e-3)
    P = oracle_lib.Problem(path)
    t, d, c = make(path, 32, batch=batch)
    rng = np.random.default_rng(6)
    r = (rng.standard_normal(P.size) * np.exp(rng.uniform(-3, 3, P.size))).astype(np.float32).astype(np.float64)
    mr = (r + 0.3 * rng.standard_normal(P.size)).astype(np.float32).astype(np.float64)
    out = np.zeros(3)
    from spock_gb300 import _p
    assert sg.lib().spock_reduce_check(c._h, _p(r), _p(mr), _p(out)) == 0, sg.lib().spock_last_error()
    ref = np.array([r @ mr, np.abs(mr).max(), r @ r])
    assert out[1] == ref[1]
    assert abs(out[0] - ref[0]) <= 1e-6 * np.abs(r * mr).sum()
    assert abs(out[2] - ref[2]) <= 1e-6 * ref[2]


@pytest.fixture(scope="module")
def bench_resolves(oracle_lib, tmp_problems):
    """The benchmark problem (config 2, costs x 1e-3), 32 instances at the FP64 oracle's cold
    solutions z0, and the oracle's re-solves zr after an x0 disturbance U[-0.05, 0.05]^50 (tol
    1e-4, Anderson memory 5).  Shared by the tests below: the oracle's solves take minutes."""
    from spock_gb300 import configs
    path, x0 = configs.cached("config2", tmp_problems, seed=0, count=32, cost_scale=1e-3)
    P = oracle_lib.Problem(path)
    opts = oracle_lib.options(tol=1e-4, anderson=5, max_iters=20000)
    z0 = np.zeros((32, P.size))
    _, st, _, _, _ = P.solve_many_warm(x0, z0, opts, 16, warm=False)
    assert (st == 0).all()
    x1 = np.clip(x0 + np.random.default_rng(3).uniform(-.05, .05, x0.shape), -1, 1)
    zr = z0.copy()
    _, st, its, _, _ = P.solve_many_warm(x1, zr, opts, 16, warm=True)
    assert (st == 0).all()
    return path, P, x1, z0, zr, its


def test_fp32_bench_workload_against_fp64_oracle(bench_resolves):
    """The benchmark's step on its problem (config 2, costs x 1e-3): 32 instances at the FP64
    oracle's cold solutions are re-solved after an x0 disturbance U[-0.05, 0.05]^50 to tol(1e-4),
    by the FP32 batched solver on the GPU and by the FP64 oracle from the same starting point.
    Both converge; the GPU's optimal costs s_0 are within 1e-2 (relative) and its first inputs u_0
    within 1e-2 of the oracle's -- two stopping points of the same iteration at the same
    tolerance, in FP32 and FP64 (the benchmark line reports the measured errors as fp64_error)."""
    path, P, x1, z0, zr, _ = bench_resolves
    t, d, c = make(path, 32, batch=32, tol=1e-4, max_iters=20000, anderson=5)
    assert (c.runSpockBatch(x1, prev=z0) == 0).all()
    oS = P.size_prim - P.n
    zg = c.solutions()
    cost_err = np.abs(zg[:, oS] - zr[:, oS]) / np.abs(zr[:, oS])
    ug, ur = zg[:, :P.nu] / P.scaling[P.nx:P.nx + P.nu], zr[:, :P.nu] / P.scaling[P.nx:P.nx + P.nu]
    print(f"FP32 vs FP64 at tol(1e-4): cost {cost_err.max():.3g} (max), u0 {np.abs(ug - ur).max():.3g} (max)")
    assert cost_err.max() <= 1e-2 and np.abs(ug - ur).max() <= 1e-2


def test_fp64_finish_of_the_bench_workload(bench_resolves):
    """The FP64 finish (spock_set_fp64_finish) on the benchmark's step: 64 instances (the 32
    re-solves of the test above, each twice) start in FP32; after 20 rounds, once at most 32 are
    running, those continue the same iteration in FP64 with their whole SuperMann state.  All
    converge, both copies of an instance end identical (the move keeps slots apart), the
    iteration counters run on across the move, and the optimal costs and first inputs agree with
    the FP64 oracle's re-solves to 1e-2 as for the plain FP32 solve."""
    path, P, x1, z0, zr, its_ref = bench_resolves
    t, d, c = make(path, 32, batch=64, tol=1e-4, max_iters=20000, anderson=5)
    c.fp64Finish(20)
    assert (c.runSpockBatch(x1, prev=z0) == 0).all()
    zg = c.solutions()
    assert np.array_equal(zg[:32], zg[32:])
    iters = c.countersAll()[:, 6]
    assert np.array_equal(iters[:32], iters[32:]) and iters.max() > 20
    oS = P.size_prim - P.n
    zr2 = np.concatenate((zr, zr))
    cost_err = np.abs(zg[:, oS] - zr2[:, oS]) / np.abs(zr2[:, oS])
    scale_u = P.scaling[P.nx:P.nx + P.nu]
    u_err = np.abs(zg[:, :P.nu] / scale_u - zr2[:, :P.nu] / scale_u).max()
    print(f"FP32 + FP64 finish vs FP64 at tol(1e-4): cost {cost_err.max():.3g} (max), u0 {u_err:.3g} (max); "
          f"outer iterations mean {iters.mean():.1f} max {iters.max()} (oracle mean {its_ref.mean():.1f} "
          f"max {its_ref.max()})")
    assert cost_err.max() <= 1e-2 and u_err <= 1e-2
