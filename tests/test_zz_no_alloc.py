"""The allocation-free dynamics projection (spock_project_dynamics_noalloc).

Callers that cannot allocate device memory while they solve (a control loop re-solving under
a hard deadline, or a host whose framework owns the device memory pool) use this entry point:
it keeps the projection's workspaces in a static device buffer.  Its result must equal the
dynamics projection inside the existing spock_cp_step: with a zero dual part, T(z) leaves
(u, x) equal to the projection of z's (u, x).  Checked twice in a row on each problem,
FP64 to 1e-12 and FP32 to 2e-5 relative (the operator tolerances of test_gpu_parity.py).
This file is collected last on purpose.
"""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden

import spock_gb300 as sg

pytestmark = pytest.mark.gpu


def _solver(case, precision):
    t = sg.ScenarioTree(os.path.join(GOLDEN, case))
    d = sg.ProblemData(t)
    return t, d, sg.CacheBuilder(t, d).precision(precision).batch(1).build()


@pytest.mark.parametrize("case,precision,tol", [("cfg1", 64, 1e-12), ("qpl", 64, 1e-12), ("qpl", 32, 2e-5)])
def test_no_alloc_projection_matches_cp_step(case, precision, tol):
    torch = pytest.importorskip("torch")
    sg.build()
    t, d, c = _solver(case, precision)
    nx, nu, n, nnl = t.numStates(), t.numInputs(), t.numNodes(), t.numNonleafNodes()
    head = nu * nnl + nx * n
    dt = torch.float64 if precision == 64 else torch.float32
    x0 = golden(case, "initialState_d.bt")
    x0s = torch.tensor(x0 * d.scaling()[:nx], dtype=dt, device="cuda")
    rng = np.random.default_rng(17)
    side = torch.cuda.Stream()
    for call in range(2):  # two calls in a row share the static workspace
        z = np.zeros(c.sizeIterate())
        z[:head] = 3 * rng.standard_normal(head)
        ref = c.cpStep(x0, z)[:head]  # existing entry point
        buf = torch.tensor(z[:head], dtype=dt, device="cuda")
        torch.cuda.synchronize()
        # the second call runs on a caller-created stream, and device memory in use must not
        # change across it (the first call may load the library's module holding the static
        # buffer: with lazy module loading the CUDA runtime places the buffer then)
        stream = None if call == 0 else ctypes.c_void_p(side.cuda_stream)
        free_before = torch.cuda.mem_get_info()[0]
        rc = sg.lib().spock_project_dynamics_noalloc(c._h, ctypes.c_void_p(x0s.data_ptr()),
                                                      ctypes.c_void_p(buf.data_ptr()), stream)
        free_after = torch.cuda.mem_get_info()[0]
        assert rc == 0, sg.lib().spock_last_error().decode()
        if call > 0:
            assert free_after == free_before, (free_before, free_after)
        torch.cuda.synchronize()
        out = buf.cpu().double().numpy()
        assert np.abs(out - ref).max() <= tol * max(1., np.abs(ref).max()), call


def test_no_alloc_rejects_batched_solver():
    pytest.importorskip("torch")
    t = sg.ScenarioTree(os.path.join(GOLDEN, "cfg1"))
    d = sg.ProblemData(t)
    c = sg.CacheBuilder(t, d).batch(2).build()
    rc = sg.lib().spock_project_dynamics_noalloc(c._h, ctypes.c_void_p(1), ctypes.c_void_p(1), None)
    assert rc == 1 and b"batch 1" in sg.lib().spock_last_error()


def test_no_alloc_projection_in_a_captured_graph():
    """The call on a capturing stream launches without waiting, so it can be recorded into a
    CUDA graph; replaying the graph gives the same projection as a direct call."""
    torch = pytest.importorskip("torch")
    t, d, c = _solver("cfg1", 64)
    nx, nu, n, nnl = t.numStates(), t.numInputs(), t.numNodes(), t.numNonleafNodes()
    head = nu * nnl + nx * n
    x0s = torch.tensor(golden("cfg1", "initialState_d.bt") * d.scaling()[:nx], dtype=torch.float64, device="cuda")
    z = torch.tensor(3 * np.random.default_rng(5).standard_normal(head), dtype=torch.float64, device="cuda")
    direct = z.clone()
    call = lambda buf, stream: sg.lib().spock_project_dynamics_noalloc(
        c._h, ctypes.c_void_p(x0s.data_ptr()), ctypes.c_void_p(buf.data_ptr()), stream)
    assert call(direct, None) == 0, sg.lib().spock_last_error().decode()
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    buf = torch.empty_like(z)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=side):
        rc = call(buf, ctypes.c_void_p(side.cuda_stream))
    assert rc == 0, sg.lib().spock_last_error().decode()
    for _ in range(2):
        buf.copy_(z)
        g.replay()
        torch.cuda.synchronize()
        assert torch.equal(buf, direct)
