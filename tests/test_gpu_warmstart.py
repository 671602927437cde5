"""Learned warm start (config 5): the MLP kernels against an FP64 numpy restatement, and the
PCA + MLP warm start run end to end."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

import spock_gb300 as sg

pytestmark = pytest.mark.gpu


def bf16(a):
    """Round float32 to bfloat16 (nearest, ties to even), as __float2bfloat16 does."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return u.view(np.float32).astype(np.float64)


def gelu(a):
    c = np.sqrt(2. / np.pi)
    t = np.tanh(c * (a + 0.044715 * a ** 3))
    return 0.5 * a * (1. + t), 0.5 * (1. + t) + 0.5 * a * (1. - t * t) * c * (1. + 3 * 0.044715 * a * a)


def unpack(p, dims):
    out, o = [], 0
    for l in range(3):
        W = p[o:o + dims[l + 1] * dims[l]].reshape((dims[l + 1], dims[l]), order="F").astype(np.float64)
        o += dims[l + 1] * dims[l]
        b = p[o:o + dims[l + 1]].astype(np.float64)
        o += dims[l + 1]
        out.append((W, b))
    return out


def test_mlp_forward_and_gradients_match_numpy():
    import torch
    from spock_gb300.warmstart import Mlp
    sg.build()
    dims = (5, 33, 17, 4)
    m = Mlp(dims, seed=1)
    p, _ = m.params()
    rng = np.random.default_rng(0)
    X = rng.standard_normal((70, dims[0])).astype(np.float32)
    T = rng.standard_normal((70, dims[3])).astype(np.float32)
    xt, tt = torch.tensor(X, device="cuda"), torch.tensor(T, device="cuda")
    loss = m.train_step(xt, tt, 0.)  # gradients only
    _, g = m.params()
    (W1, b1), (W2, b2), (W3, b3) = unpack(p, dims)
    Xc = X.T.astype(np.float64)
    A1 = bf16(W1) @ Xc + b1[:, None]
    H1, d1 = gelu(A1)
    A2 = bf16(W2) @ H1 + b2[:, None]
    H2, d2 = gelu(A2)
    Y = bf16(W3) @ H2 + b3[:, None]
    R = Y - T.T
    ref_loss = (R ** 2).mean()
    dY = 2 * R / R.size
    dA2 = (bf16(W3).T @ dY) * d2
    dA1 = (bf16(W2).T @ dA2) * d1
    ref = np.concatenate([(dA1 @ Xc.T).ravel(order="F"), dA1.sum(1), (dA2 @ H1.T).ravel(order="F"), dA2.sum(1),
                          (dY @ H2.T).ravel(order="F"), dY.sum(1)])
    assert abs(loss - ref_loss) <= 1e-4 * ref_loss
    assert np.abs(g - ref).max() <= 1e-4 * np.abs(ref).max()
    y = m.forward(xt).cpu().numpy()
    assert np.abs(y - Y.T).max() <= 1e-4 * max(1., np.abs(Y).max())
    # one Adam step lowers the loss on this batch
    l0 = m.train_step(xt, tt, 1e-2)
    assert m.train_step(xt, tt, 0.) < l0


def test_learned_warm_start_end_to_end(oracle_lib):
    """Fit PCA + MLP on 256 solved instances of the reference's test problem, predict warm starts
    for 64 new initial states: every warm-started instance converges to the same first input as
    a cold solve (the warm start changes the path, not the answer)."""
    import torch
    from spock_gb300.warmstart import PcaMlpWarmStart
    path = os.path.join(GOLDEN, "reftest")
    P = oracle_lib.Problem(path)
    rng = np.random.default_rng(9)
    # x0 = 1.1 + s (1, 1, 1), s in [-0.05, 0.05]: feasible for the problem's terminal box |x| <= 0.1
    xtr = 1.1 + rng.uniform(-.05, .05, (256, 1)) * np.ones(P.nx)
    t = sg.ScenarioTree(path)
    d = sg.ProblemData(t)
    c = sg.CacheBuilder(t, d).tol(1e-4).andersonBuffer(3).maxIters(20000).precision(64).batch(256).build()
    assert (c.runSpockBatch(xtr) == 0).all()
    zs = torch.tensor(c.solutions(), dtype=torch.float32, device="cuda")
    ws = PcaMlpWarmStart(k=8, hidden=64, seed=2)
    losses = ws.fit(xtr, zs, epochs=60, batch=64, lr=3e-3)
    assert losses[-1] < losses[0]
    xte = 1.1 + rng.uniform(-.05, .05, (64, 1)) * np.ones(P.nx)
    cw = sg.CacheBuilder(t, d).tol(1e-4).andersonBuffer(3).maxIters(20000).precision(64).batch(64).build()
    ws.warm_start(cw, xte)
    assert (cw.resolveBatch(xte) == 0).all()
    cc = sg.CacheBuilder(t, d).tol(1e-4).andersonBuffer(3).maxIters(20000).precision(64).batch(64).build()
    assert (cc.runSpockBatch(xte) == 0).all()
    u_w, u_c = cw.firstInputs(), cc.firstInputs()
    assert np.abs(u_w - u_c).max() <= 5e-2 * max(1., np.abs(u_c).max())


def test_learned_warm_start_gain():
    """What the learned start gains (config 1's problem and tolerance 1e-3): trained on 1,024 cold
    solves, it reaches the absolute tolerance on 256 held-out initial states in fewer mean outer
    iterations than a cold start and than a start from the previous held-out instance's solution
    (the shifted previous solution of a stream of requests); every start converges."""
    import torch
    from spock_gb300.warmstart import PcaMlpWarmStart
    path = os.path.join(GOLDEN, "cfg1")
    t = sg.ScenarioTree(path)
    d = sg.ProblemData(t)
    rng = np.random.default_rng(4)
    xtr = rng.uniform(-1, 1, (1024, t.numStates()))
    xte = rng.uniform(-1, 1, (256, t.numStates()))
    ctr = sg.CacheBuilder(t, d).tol(1e-3).andersonBuffer(3).maxIters(20000).precision(32).batch(1024).build()
    assert (ctr.runSpockBatch(xtr) == 0).all()
    ws = PcaMlpWarmStart(k=64, hidden=256, seed=0)
    ws.fit(xtr, torch.tensor(ctr.solutions(), dtype=torch.float32, device="cuda"), epochs=300, batch=256, lr=1e-3)

    def absolute():
        return (sg.CacheBuilder(t, d).toleranceAbsolute(1e-3).toleranceRelative(0.).andersonBuffer(3).maxIters(20000)
                .precision(32).batch(256).build())
    cold = absolute()
    assert (cold.runSpockBatch(xte) == 0).all()
    learned = absolute()
    ws.warm_start(learned, xte)
    pred = ws.predict(xte).double().cpu().numpy()  # the same iterate by a torch product
    assert np.abs(learned.solutions() - pred).max() <= 1e-4 * np.abs(pred).max()
    assert (learned.resolveBatch(xte) == 0).all()
    prev = absolute()
    z = torch.roll(torch.tensor(cold.solutions(), dtype=torch.float32, device="cuda"), 1, 0).T.contiguous()
    prev.setIterateDevice(z.data_ptr(), 32)
    assert (prev.resolveBatch(xte) == 0).all()
    it = {k: c.solveIters().mean() for k, c in (("cold", cold), ("learned", learned), ("previous", prev))}
    print("mean outer iterations", it)
    assert it["learned"] < it["cold"] and it["learned"] < it["previous"], it
