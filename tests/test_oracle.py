"""The FP64 CPU oracle against the reference's own fixtures and literal known answers.

Fixtures: tests/golden/<case>/ written by the reference's Python factory (make_golden.py).
Literal answers: tests/cuda/testProjections.cu (SOC), testKernels.cu (box), testRisks.cu
(AVaR index pattern), testTree.cu (tree sizes) of ruairimoran/spock.cu.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, GOLDEN_CASES, golden


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_operator_fixtures(oracle_lib, case):
    """L and L* reproduce the reference's op/adj fixtures (testOperator.cu:38-86)."""
    P = oracle_lib.Problem(os.path.join(GOLDEN, case))
    prim = golden(case, "test_primBeforeOp_d.bt")
    dual = golden(case, "test_dualAfterOpBeforeAdj_d.bt")
    assert np.allclose(P.op(prim), dual, rtol=0, atol=1e-10)
    assert np.allclose(P.adj(dual), golden(case, "test_primAfterAdj_d.bt"), rtol=0, atol=1e-10)


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_adjoint_identity(oracle_lib, case):
    """<L x, y> = <x, L* y> (testOperator.cu:93-113) on the reference's random pair."""
    P = oracle_lib.Problem(os.path.join(GOLDEN, case))
    x = golden(case, "test_adjRandomPrim_d.bt")
    y = golden(case, "test_adjRandomDual_d.bt")
    ref = golden(case, "test_adjRandomResult_d.bt")[0]
    uno, dos = y @ P.op(x), P.adj(y) @ x
    assert abs(uno - dos) <= 1e-9 * abs(uno)
    assert abs(uno - ref) <= 1e-9 * abs(ref)


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_dot_m_fixture(oracle_lib, case):
    """x' M x against the reference's dotM fixture (testCache.cu:206-221)."""
    P = oracle_lib.Problem(os.path.join(GOLDEN, case))
    v = golden(case, "test_dotVector_d.bt")
    ref = golden(case, "test_dotResult_d.bt")[0]
    assert abs(P.dot_m(v, v) - ref) <= 1e-9 * abs(ref)


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_step_size(oracle_lib, case):
    """0.99 / ||L|| by power iteration matches the ARPACK value in data.json (problem.py:402-417)."""
    P = oracle_lib.Problem(os.path.join(GOLDEN, case))
    assert abs(.99 / np.sqrt(P.norm_L_sq(20000)) - P.step) <= 1e-9 * P.step


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_offline_cache(oracle_lib, case):
    """Riccati-like dynamics cache and AVaR nullspace projectors (problem.py:192-231)."""
    P = oracle_lib.Problem(os.path.join(GOLDEN, case))
    got = P.offline_dynamics(golden(case, "dynamics_AB_d.bt"))
    for arr, name in zip(got, ["P", "K", "lowCholesky", "ABKTr", "APB"]):
        ref = golden(case, f"dynamics_{name}_d.bt")
        assert np.allclose(arr, ref, rtol=0, atol=1e-11 * max(1., np.abs(ref).max())), name
    alpha = json.load(open(os.path.join(GOLDEN, case, "data.json")))["risk"]["alpha"]
    nn = golden(case, "risk_NNtr_d.bt").reshape(P.nnl, -1)
    for i in range(P.nnl):
        assert np.allclose(P.offline_kernel(alpha, i), nn[i], atol=1e-12)


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_kernel_projection_membership(oracle_lib, case):
    """Projected (y, t[ch], s[ch]) lies in ker S2 and the projection is idempotent
    (testCache.cu:58-113, 121-199)."""
    P = oracle_lib.Problem(os.path.join(GOLDEN, case))
    rng = np.random.default_rng(1)
    S2 = golden(case, "test_S2_d.bt").reshape(P.nnl, P.nulldim, P.ne).transpose(0, 2, 1)
    y = rng.uniform(-100, 100, P.ydim * P.nnl)
    t = rng.uniform(-100, 100, P.n)
    s = rng.uniform(-100, 100, P.n)
    y1, t1, s1 = P.project_kernel(y, t, s)
    ch_from = golden(case, "childrenFrom_u.bt").astype(np.int64)
    num_ch = golden(case, "numChildren_u.bt").astype(np.int64)
    for i in range(P.nnl):
        v = np.zeros(P.nulldim)
        v[:P.ydim] = y1[i * P.ydim:(i + 1) * P.ydim]
        c0, nc = ch_from[i], num_ch[i]
        v[P.ydim:P.ydim + nc] = t1[c0:c0 + nc]
        v[P.ydim + P.ne:P.ydim + P.ne + nc] = s1[c0:c0 + nc]
        assert np.abs(S2[i] @ v).max() <= 1e-9 * np.abs(v).max()
    y2, t2, s2 = P.project_kernel(y1, t1, s1)
    assert np.allclose(y2, y1, atol=1e-9) and np.allclose(t2, t1, atol=1e-9) and np.allclose(s2, s1, atol=1e-9)


def test_soc_literal_values(oracle_lib):
    """Three 5-D cones, expected values of testProjections.cu:146-170."""
    socs = [1., 2., 3., 4., .5, 5., 6., 7., 8., -200, 9., -10., 11., -12., 100]
    expected = [0.5456435464587639, 1.0912870929175278, 1.6369306393762917, 2.1825741858350556,
                2.988612787525831, 0., 0., 0., 0., 0., 9., -10., 11., -12., 100.]
    assert np.allclose(oracle_lib.project_soc_columns(socs, 5), expected, atol=1e-12)


@pytest.mark.parametrize("n", [555, 1034])
def test_soc_cases_i1_i2_i3(oracle_lib, n):
    """Cases i1 (inside), i2 (polar) and i3 (else) of testProjections.cu:17-144, including a
    cone longer than one 1024-thread block."""
    a = np.zeros(n); a[-1] = 1.
    assert np.array_equal(oracle_lib.project_soc_columns(a, n), a)
    bvec = np.zeros(n); bvec[-1] = -1.
    assert np.array_equal(oracle_lib.project_soc_columns(bvec, n), np.zeros(n))
    c = np.ones(n); c[-1] = 0.
    out = oracle_lib.project_soc_columns(c, n)
    assert np.linalg.norm(out[:-1]) <= out[-1] * (1 + 1e-12)


def test_box_projection(oracle_lib):
    """testKernels.cu:14-35: 1025 entries, +-inf bounds at index 0."""
    n, ub, oob = 1025, 4., .1
    v = np.full(n, ub + oob)
    v[::2] *= -1
    v[::3] *= .5
    lb = np.full(n, -ub)
    ubv = np.full(n, ub)
    lb[0], ubv[0] = -np.inf, np.inf
    out = oracle_lib.project_box(v, lb, ubv)
    assert abs(out[0] - (-(ub + oob) * .5)) < 1e-12
    assert (out >= -ub).all() and (out <= ub).all()


def test_avar_index_pattern(oracle_lib):
    """testRisks.cu:39-50: on the reference test tree only these entries of a -10 vector survive
    the AVaR dual-cone projection."""
    P = oracle_lib.Problem(os.path.join(GOLDEN, "reftest"))
    dual = np.zeros(P.size_dual)
    dual[:P.ydim * P.nnl] = -10.
    out = P.project_dual(dual)[:P.ydim * P.nnl]
    expected = np.zeros(P.ydim * P.nnl)
    expected[[4, 9, 14, 17, 18, 19, 22, 23, 24, 27, 28, 29, 32, 33, 34]] = -10.
    assert np.array_equal(out, expected)


def test_tree_fixture_sizes(oracle_lib):
    """testTree.cu:43-46: numEvents=2, nonleaf=7, nodes=11, stages=4."""
    P = oracle_lib.Problem(os.path.join(GOLDEN, "reftest"))
    assert (P.ne, P.nnl, P.n, P.ns) == (2, 7, 11, 4)


@pytest.mark.parametrize("case,x0", [("reftest", None), ("cfg1", "file"), ("qpl", "file")])
@pytest.mark.parametrize("algo", ["spock", "cp"])
def test_convergence(oracle_lib, case, x0, algo):
    """runSpock / runCp reach status 0 at tol 1e-3 within 1500 iterations (testCache.cu:279-308)."""
    P = oracle_lib.Problem(os.path.join(GOLDEN, case))
    x = np.full(P.nx, 1.1) if x0 is None else golden(case, "initialState_d.bt")
    z, st = P.run(x, oracle_lib.options(tol=1e-3, max_iters=1500 if algo == "spock" else 5000), algo)
    assert st.status == 0


def test_spock_and_cp_agree(oracle_lib):
    """Two different algorithms (SuperMann and plain CP) reach the same minimiser: the first
    input and the optimal value s_0 agree at tight tolerance (reference test problem)."""
    P = oracle_lib.Problem(os.path.join(GOLDEN, "reftest"))
    x0 = np.full(P.nx, 1.1)
    z1, s1 = P.run(x0, oracle_lib.options(tol=1e-10, max_iters=20000), "spock")
    z2, s2 = P.run(x0, oracle_lib.options(tol=1e-10, max_iters=200000), "cp")
    assert s1.status == 0 and s2.status == 0
    _, u1 = P.states_inputs(z1)
    _, u2 = P.states_inputs(z2)
    assert np.allclose(u1[:P.nu], u2[:P.nu], atol=1e-7)
    s0 = P.size_prim - P.n
    assert abs(z1[s0] - z2[s0]) <= 1e-6 * abs(z2[s0])


def test_input_ball_projection(oracle_lib, tmp_problems):
    """RectangleInputBall (the second-order-cone input constraint ||u||_2 <= r): after the dual
    projection every nonleaf node's u rows lie in the ball, rows inside it are unchanged, and the
    x rows are clamped to their box (the root's states are free)."""
    from spock_gb300 import configs
    path, _ = configs.cached("config3", tmp_problems, seed=1, count=1, nx=4, nu=3, horizon=3, stopping=2,
                             events=2, radius=.5)
    P = oracle_lib.Problem(path)
    rng = np.random.default_rng(3)
    d = 2 * rng.standard_normal(P.size_dual)
    out = P.project_dual(d)
    nxu = P.nx + P.nu
    oIII = P.ydim * P.nnl + P.nnl
    for i in range(P.nnl):
        u0 = d[oIII + i * nxu + P.nx:oIII + (i + 1) * nxu]
        u1 = out[oIII + i * nxu + P.nx:oIII + (i + 1) * nxu]
        n0 = np.linalg.norm(u0)
        assert np.linalg.norm(u1) <= .5 + 1e-12
        assert np.allclose(u1, u0 if n0 <= .5 else u0 * .5 / n0, atol=1e-14)
        x1 = out[oIII + i * nxu:oIII + i * nxu + P.nx]
        if i > 0:
            assert (np.abs(x1) <= 3 + 1e-12).all()


def test_fp32_emulation_modes(oracle_lib):
    """The oracle's FP32 emulation (spock_oracle.h, OR_EMU_*): under the GPU-like mode a CP step
    returns float-representable values within single-precision distance of the FP64 step; the
    forward-rollout remedies keep that; switching back to mode 0 restores FP64 bit for bit."""
    path = os.path.join(GOLDEN, "cfg1")
    P = oracle_lib.Problem(path)
    rng = np.random.default_rng(8)
    z = rng.standard_normal(P.size)
    x0s = rng.uniform(-1, 1, P.nx) * P.scaling[:P.nx]
    a = P.cp_step(x0s, z)
    try:
        for mode in (oracle_lib.EMU_GPU_FP32, oracle_lib.EMU_GPU_FP32 | oracle_lib.EMU_FWD64,
                     oracle_lib.EMU_GPU_FP32 | oracle_lib.EMU_FWDC, oracle_lib.EMU_GPU_FP32 | oracle_lib.EMU_FWDCX,
                     oracle_lib.EMU_GPU_FP32 | oracle_lib.EMU_FWDK):
            oracle_lib.set_emulation(mode)
            b = oracle_lib.Problem(path).cp_step(x0s.astype(np.float32).astype(np.float64),
                                                 z.astype(np.float32).astype(np.float64))
            assert np.array_equal(b, b.astype(np.float32).astype(np.float64))
            assert 0 < np.abs(b - a).max() <= 1e-4 * np.abs(a).max()
    finally:
        oracle_lib.set_emulation(0)
    assert np.array_equal(P.cp_step(x0s, z), a)


def test_fp32_emulation_forward_rollout(oracle_lib, tmp_problems):
    """On a config-2 sized problem (607 nodes, nx=50), the dynamics projection's deviation from
    FP64 arithmetic on the same float data: float accumulation everywhere gives the largest; a
    forward rollout accumulated in double or with Dot2 compensation cuts it; plain float storage
    alone is smallest."""
    from spock_gb300 import configs
    path, x0 = configs.cached("config2", tmp_problems, seed=0, count=1, cost_scale=1e-3)
    rng = np.random.default_rng(0)
    P0 = oracle_lib.Problem(path)
    x = rng.standard_normal(P0.nx * P0.n)
    u = rng.standard_normal(P0.nu * P0.nnl)
    x0s = (x0[0] * P0.scaling[:P0.nx]).astype(np.float32).astype(np.float64)
    D, A, V = oracle_lib.EMU_DATA, oracle_lib.EMU_ACC, oracle_lib.EMU_VEC
    err = {}
    try:
        oracle_lib.set_emulation(D)
        ref = np.concatenate(oracle_lib.Problem(path).project_dynamics(x0s, x, u))
        for name, mode in [("acc", D | A | V), ("fwd64", D | A | V | oracle_lib.EMU_FWD64),
                           ("dot2", D | A | V | oracle_lib.EMU_FWDC), ("vec", D | V)]:
            oracle_lib.set_emulation(mode)
            out = np.concatenate(oracle_lib.Problem(path).project_dynamics(x0s, x, u))
            err[name] = np.abs(out - ref).max() / np.abs(ref).max()
    finally:
        oracle_lib.set_emulation(0)
    assert err["vec"] < err["dot2"] < err["acc"] and err["fwd64"] < err["acc"]
    assert err["acc"] < 1e-5 and err["dot2"] < 0.6 * err["acc"]


def test_fp32_emulation_backward_sweep(oracle_lib, tmp_problems):
    """With the forward rollout compensated (Dot2, as on the GPU), the rest of the dynamics
    projection's deviation from FP64 on a config-2 sized problem comes from the backward sweep's
    float accumulation: accumulating that sweep exactly (OR_EMU_ACCX_BACK) halves it, while the
    scope of L and L* (OR_EMU_ACCX_OPS) does not touch the projection."""
    from spock_gb300 import configs
    path, x0 = configs.cached("config2", tmp_problems, seed=0, count=1, cost_scale=1e-3)
    rng = np.random.default_rng(0)
    P0 = oracle_lib.Problem(path)
    x = rng.standard_normal(P0.nx * P0.n)
    u = rng.standard_normal(P0.nu * P0.nnl)
    x0s = (x0[0] * P0.scaling[:P0.nx]).astype(np.float32).astype(np.float64)
    gpu = oracle_lib.EMU_DATA | oracle_lib.EMU_ACC | oracle_lib.EMU_VEC | oracle_lib.EMU_FWDC
    err = {}
    try:
        oracle_lib.set_emulation(oracle_lib.EMU_DATA)
        ref = np.concatenate(oracle_lib.Problem(path).project_dynamics(x0s, x, u))
        for name, mode in [("dot2", gpu), ("back", gpu | oracle_lib.EMU_ACCX_BACK),
                           ("ops", gpu | oracle_lib.EMU_ACCX_OPS)]:
            oracle_lib.set_emulation(mode)
            out = np.concatenate(oracle_lib.Problem(path).project_dynamics(x0s, x, u))
            err[name] = np.abs(out - ref).max() / np.abs(ref).max()
    finally:
        oracle_lib.set_emulation(0)
    assert err["back"] < 0.6 * err["dot2"] and err["ops"] == err["dot2"], err
