"""The tcgen05 BF16 GEMM (csrc/umma_gemm.cu: TMA-staged operands, tcgen05.mma into tensor memory,
FP32 accumulation) against an FP64 PyTorch product of the same BF16 operands, and the learned
warm start's reconstruction, which writes mean + basis coef' into an FP32 solver's iterate."""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN

import spock_gb300 as sg

pytestmark = pytest.mark.gpu


def _gelu(a):
    return 0.5 * a * (1 + np.tanh(0.7978845608028654 * (a + 0.044715 * a ** 3)))


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (300, 200, 192), (1000, 77, 128), (64, 1100, 1024)])
def test_gemm_matches_fp64_product(M, N, K):
    torch = pytest.importorskip("torch")
    sg.build()
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    ra = torch.randn(M, device="cuda", generator=g)
    ca = torch.randn(N, device="cuda", generator=g)
    ldd = N + 3
    D = torch.full((M, ldd), 7.0, device="cuda")
    Dact = torch.full((M, ldd), 7.0, device="cuda")
    vp = ctypes.c_void_p
    for call in range(2):
        rc = sg.lib().spock_gemm_bf16(vp(A.data_ptr()), vp(B.data_ptr()), M, N, K, 0.5, vp(ra.data_ptr()),
                                      vp(ca.data_ptr()), 1, vp(D.data_ptr()), vp(Dact.data_ptr()), ldd, 0)
        assert rc == 0, sg.lib().spock_last_error().decode()
        ref = (0.5 * (A.double() @ B.double().T) + ra.double()[:, None] + ca.double()[None, :]).cpu().numpy()
        out = D[:, :N].double().cpu().numpy()
        assert np.abs(out - ref).max() <= 1e-5 * np.abs(ref).max(), call
        assert np.abs(Dact[:, :N].double().cpu().numpy() - _gelu(ref)).max() <= 1e-5 * np.abs(ref).max()
        assert (D[:, N:] == 7.0).all()  # nothing written past column N


def test_gemm_rejects_bad_k():
    torch = pytest.importorskip("torch")
    A = torch.zeros(128, 96, device="cuda", dtype=torch.bfloat16)
    D = torch.zeros(128, 128, device="cuda")
    vp = ctypes.c_void_p
    rc = sg.lib().spock_gemm_bf16(vp(A.data_ptr()), vp(A.data_ptr()), 128, 128, 96, 1.0, None, None, 0,
                                  vp(D.data_ptr()), None, 128, 0)
    assert rc != 0 and b"multiple of 64" in sg.lib().spock_last_error()


def test_warm_start_reconstruction_writes_iterate():
    torch = pytest.importorskip("torch")
    t = sg.ScenarioTree(os.path.join(GOLDEN, "cfg1"))
    d = sg.ProblemData(t)
    B, k = 64, 64
    c = sg.CacheBuilder(t, d).precision(32).batch(B).build()
    n = c.sizeIterate()
    g = torch.Generator(device="cuda").manual_seed(3)
    basis = torch.randn(n, k, device="cuda", generator=g).to(torch.bfloat16)
    coef = torch.randn(B, k, device="cuda", generator=g).to(torch.bfloat16)
    mean = torch.randn(n, device="cuda", generator=g)
    vp = ctypes.c_void_p
    rc = sg.lib().spock_warm_start_pca(c._h, vp(basis.data_ptr()), vp(coef.data_ptr()), k, vp(mean.data_ptr()))
    assert rc == 0, sg.lib().spock_last_error().decode()
    ref = (mean.double()[None, :] + coef.double() @ basis.double().T).cpu().numpy()
    z = c.solutions()
    assert np.abs(z - ref).max() <= 1e-5 * np.abs(ref).max()
    c64 = sg.CacheBuilder(t, d).precision(64).batch(B).build()  # FP64 solvers get the FP32 sums widened
    assert sg.lib().spock_warm_start_pca(c64._h, vp(basis.data_ptr()), vp(coef.data_ptr()), k,
                                         vp(mean.data_ptr())) == 0
    assert np.abs(c64.solutions() - ref).max() <= 1e-5 * np.abs(ref).max()
