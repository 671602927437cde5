"""Learned warm start for batches of one problem family (no counterpart in the reference).

A three-layer MLP (x0 -> 1024 -> 1024 -> k, GELU, BF16 weights, FP32 accumulation) predicts the
coefficients of a k-dimensional PCA basis of primal-dual solutions that the solver itself
generated; the predicted iterate mean + basis @ coefficients is handed to the solver on the device
(spock_set_iterate_device) and every instance is then solved to the same tolerance as a cold
start, so the warm start changes the iteration count, never the answer.

The MLP's forward, backward and Adam kernels are the library's own (csrc/mlp.cu, spock_mlp_*),
all products on the tcgen05 tensor cores.  The reconstruction mean + basis coef' is the
library's tensor-core GEMM as well (spock_warm_start_pca), writing the solver's iterate directly;
basis and coefficients enter as BF16 hi + lo pairs (three K segments), so the reconstructed
iterate is accurate to about FP32.  The PCA basis itself is computed once, offline, with a
randomized range finder whose products are plain library GEMMs (torch.matmul) and an SVD of the
small projected matrix.
"""
import ctypes

import numpy as np

from . import _check, _ip, lib

_fp = ctypes.POINTER(ctypes.c_float)


class Mlp:
    """spock_mlp: dims = (inputs, hidden, hidden, outputs)."""

    def __init__(self, dims, device=0, seed=0):
        self.dims = tuple(int(d) for d in dims)
        d = np.array(self.dims, dtype=np.int32)
        h = ctypes.c_void_p()
        _check(lib().spock_mlp_create(d.ctypes.data_as(_ip), device, ctypes.byref(h)))
        self._h = h
        self.n = int(lib().spock_mlp_param_count(h))
        rng = np.random.default_rng(seed)
        p = np.zeros(self.n, dtype=np.float32)
        o = 0
        for l in range(3):  # He-style initialisation of W, zero biases
            fan_in, fan_out = self.dims[l], self.dims[l + 1]
            p[o:o + fan_out * fan_in] = rng.standard_normal(fan_out * fan_in) * np.sqrt(2. / fan_in)
            o += fan_out * fan_in + fan_out
        self.set_params(p)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().spock_mlp_free(self._h)
            self._h = None

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.n
        _check(lib().spock_mlp_set_params(self._h, p.ctypes.data_as(_fp)))

    def params(self):
        p = np.zeros(self.n, dtype=np.float32)
        g = np.zeros(self.n, dtype=np.float32)
        _check(lib().spock_mlp_get_params(self._h, p.ctypes.data_as(_fp), g.ctypes.data_as(_fp)))
        return p, g

    def forward(self, x):
        """x: torch float32 CUDA tensor (inputs x cols, column-major = samples in columns, i.e. a
        contiguous (cols, inputs) tensor).  Returns (cols, outputs)."""
        import torch
        x = x.contiguous()
        cols = x.shape[0]
        y = torch.empty((cols, self.dims[3]), dtype=torch.float32, device=x.device)
        _check(lib().spock_mlp_forward(self._h, ctypes.c_void_p(x.data_ptr()), cols, ctypes.c_void_p(y.data_ptr())))
        return y

    def train_step(self, x, t, lr):
        x, t = x.contiguous(), t.contiguous()
        loss = ctypes.c_float()
        _check(lib().spock_mlp_train_step(self._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(t.data_ptr()),
                                          x.shape[0], float(lr), ctypes.byref(loss)))
        return loss.value


class PcaMlpWarmStart:
    """Fit on (x0, solution) pairs; predict solver iterates for new x0."""

    def __init__(self, k=128, hidden=1024, device=0, seed=0):
        self.k, self.hidden, self.device, self.seed = k, hidden, device, seed

    def fit(self, x0s, zs, epochs=200, batch=1024, lr=1e-3, oversample=32, log=None):
        """x0s: (N, nx) numpy; zs: (N, size) torch float32 CUDA tensor of solutions."""
        self.fit_basis(zs, oversample)
        return self.fit_mlp(x0s, self.project(zs), epochs, batch, lr, log)

    def fit_basis(self, zs, oversample=32):
        """Mean and k-dimensional PCA basis of solutions zs ((N, size) torch float32, CUDA)."""
        import torch
        dev = zs.device
        self.mean = zs.mean(0)
        Zc = zs - self.mean
        g = torch.Generator(device=dev).manual_seed(self.seed)
        omega = torch.randn(Zc.shape[0], self.k + oversample, device=dev, generator=g)
        Y = Zc.T @ omega                                     # (size, k + p): range of Zc'
        Q, _ = torch.linalg.qr(Y)
        _, S, Vt = torch.linalg.svd(Zc @ Q, full_matrices=False)
        self.basis = (Q @ Vt.T)[:, :self.k].contiguous()     # (size, k), orthonormal columns
        self.explained = float((S[:self.k] ** 2).sum() / (S ** 2).sum())
        self._bop = None

    def project(self, zs):
        """(N, k) coefficients of solutions zs in the basis."""
        return (zs - self.mean) @ self.basis

    def fit_mlp(self, x0s, coef, epochs=200, batch=1024, lr=1e-3, log=None):
        """Train the MLP x0 -> coefficients (coef: (N, k) torch float32, CUDA)."""
        import torch
        dev = coef.device
        g = torch.Generator(device=dev).manual_seed(self.seed + 1)
        self.cscale = coef.std(0).clamp_min(1e-12)
        self.xs_mean = torch.tensor(x0s.mean(0), dtype=torch.float32, device=dev)
        self.xs_std = torch.tensor(x0s.std(0) + 1e-12, dtype=torch.float32, device=dev)
        X = (torch.tensor(x0s, dtype=torch.float32, device=dev) - self.xs_mean) / self.xs_std
        T = coef / self.cscale
        self.mlp = Mlp((x0s.shape[1], self.hidden, self.hidden, self.k), self.device, self.seed)
        n = X.shape[0]
        losses = []
        for ep in range(epochs):
            perm = torch.randperm(n, device=dev, generator=g)
            for s in range(0, n - batch + 1, batch):
                idx = perm[s:s + batch]
                losses.append(self.mlp.train_step(X[idx], T[idx], lr))
            if log and (ep % max(1, epochs // 10) == 0 or ep == epochs - 1):
                log(f"epoch {ep}: loss {losses[-1]:.4e}")
        return losses

    def coefficients(self, x0s):
        """(B, k) torch float32 predicted basis coefficients for x0s (numpy (B, nx))."""
        import torch
        X = (torch.tensor(x0s, dtype=torch.float32, device=self.mean.device) - self.xs_mean) / self.xs_std
        return self.mlp.forward(X) * self.cscale

    def predict(self, x0s):
        """(B, size) torch float32 predicted iterates (a host-side check of warm_start)."""
        return self.mean + self.coefficients(x0s) @ self.basis.T

    def _basis_operand(self):
        """basis as a BF16 [hi | lo | hi] operand (size x 3 kP, kP = k padded to 64), built once."""
        import torch
        if getattr(self, "_bop", None) is None:
            kP = (self.k + 63) // 64 * 64
            hi = self.basis.to(torch.bfloat16)
            lo = (self.basis - hi.float()).to(torch.bfloat16)
            op = torch.zeros(self.basis.shape[0], 3 * kP, dtype=torch.bfloat16, device=self.basis.device)
            op[:, :self.k], op[:, kP:kP + self.k], op[:, 2 * kP:2 * kP + self.k] = hi, lo, hi
            self._bop, self._kP = op.contiguous(), kP
        return self._bop, self._kP

    def warm_start(self, cache, x0s):
        """Put the predicted iterates into `cache` (batch = len(x0s)) with the library's tensor-core
        GEMM; then call resolveBatch(x0s)."""
        import torch
        bop, kP = self._basis_operand()
        c = self.coefficients(x0s)
        hi = c.to(torch.bfloat16)
        lo = (c - hi.float()).to(torch.bfloat16)
        cop = torch.zeros(c.shape[0], 3 * kP, dtype=torch.bfloat16, device=c.device)
        cop[:, :self.k], cop[:, kP:kP + self.k], cop[:, 2 * kP:2 * kP + self.k] = hi, hi, lo
        mean = self.mean.float().contiguous()
        _check(lib().spock_warm_start_pca(cache._h, ctypes.c_void_p(bop.data_ptr()), ctypes.c_void_p(cop.data_ptr()),
                                          3 * kP, ctypes.c_void_p(mean.data_ptr())))
