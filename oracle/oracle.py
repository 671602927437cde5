"""ctypes binding of the FP64 CPU oracle -- TEST INFRASTRUCTURE ONLY.

The oracle (spock_oracle.c) restates the reference solver's algorithm in plain C so that the
CUDA product can be checked against it.  Only tests/, the smoke entry point and the
benchmark's CPU-baseline leg import this module; the product never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libspock_oracle.so")

_dp = ctypes.POINTER(ctypes.c_double)
_lp = ctypes.POINTER(ctypes.c_long)
_ip = ctypes.POINTER(ctypes.c_int)


class OrOptions(ctypes.Structure):
    _fields_ = [("tol_abs", ctypes.c_double), ("tol_rel", ctypes.c_double),
                ("max_time_secs", ctypes.c_double), ("max_outer", ctypes.c_long),
                ("max_inner", ctypes.c_long), ("anderson", ctypes.c_long)]


class OrStats(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("iters", ctypes.c_long), ("calls_T", ctypes.c_long),
                ("k0", ctypes.c_long), ("k1", ctypes.c_long), ("k2", ctypes.c_long),
                ("k2bt", ctypes.c_long), ("k3", ctypes.c_long), ("tol", ctypes.c_double),
                ("err", ctypes.c_double), ("seconds", ctypes.c_double)]


def build():
    """Compile the oracle with gcc (oracle/Makefile)."""
    subprocess.check_call(["make", "-s", "-C", HERE])


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.or_load.restype = ctypes.c_void_p
        L.or_load.argtypes = [ctypes.c_char_p]
        L.or_free.argtypes = [ctypes.c_void_p]
        L.or_last_error.restype = ctypes.c_char_p
        L.or_sizes.argtypes = [ctypes.c_void_p, _lp]
        L.or_step_size.restype = ctypes.c_double
        L.or_step_size.argtypes = [ctypes.c_void_p]
        L.or_scaling.argtypes = [ctypes.c_void_p, _dp]
        for f in ("or_op", "or_adj"):
            getattr(L, f).argtypes = [ctypes.c_void_p, _dp, _dp]
        L.or_project_dynamics.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.or_project_kernel.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.or_project_dual.argtypes = [ctypes.c_void_p, _dp]
        L.or_cp_step.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.or_dot_m.restype = ctypes.c_double
        L.or_dot_m.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.or_project_soc_columns.argtypes = [_dp, ctypes.c_long, ctypes.c_long]
        L.or_project_box.argtypes = [_dp, _dp, _dp, ctypes.c_long]
        for f in ("or_run_spock", "or_run_cp"):
            getattr(L, f).restype = ctypes.c_int
            getattr(L, f).argtypes = [ctypes.c_void_p, ctypes.POINTER(OrOptions), _dp, _dp, ctypes.c_int,
                                      ctypes.POINTER(OrStats)]
        L.or_states_inputs.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.or_solve_many.restype = ctypes.c_double
        L.or_solve_many.argtypes = [ctypes.c_void_p, ctypes.POINTER(OrOptions), ctypes.c_long, _dp,
                                    ctypes.c_int, _ip, _lp, _dp, _dp]
        L.or_solve_many_warm.restype = ctypes.c_double
        L.or_solve_many_warm.argtypes = [ctypes.c_void_p, ctypes.POINTER(OrOptions), ctypes.c_long, _dp,
                                         ctypes.c_int, _ip, _lp, _dp, _dp, ctypes.c_int, _lp]
        L.or_offline_dynamics.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp]
        L.or_offline_kernel.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_long, _dp]
        L.or_norm_L_sq.restype = ctypes.c_double
        L.or_norm_L_sq.argtypes = [ctypes.c_void_p, ctypes.c_long]
        L.or_set_emulation.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


# FP32 emulation modes (spock_oracle.h): problem data, matvec accumulation, vector storage,
# Anderson normal equations, and the two remedies for the forward rollout.
EMU_DATA, EMU_ACC, EMU_VEC, EMU_GRAM, EMU_FWD64, EMU_FWDC, EMU_FWDCX, EMU_FWDK = 1, 2, 4, 8, 16, 32, 64, 128
EMU_ACCX_OPS, EMU_ACCX_BACK = 256, 512  # exact accumulation in L / L*, or in the backward sweep
EMU_GPU_FP32 = EMU_DATA | EMU_ACC | EMU_VEC | EMU_GRAM


def set_emulation(mode):
    """Process-wide FP32 emulation mode (0 = plain FP64); set it before loading a Problem."""
    lib().or_set_emulation(int(mode))


def _p(a):
    return a.ctypes.data_as(_dp)


def options(tol=1e-3, tol_abs=None, tol_rel=None, max_iters=0, max_inner=8, anderson=3, max_time=0.):
    """CacheBuilder semantics: tol() sets both absolute and relative tolerance."""
    return OrOptions(tol if tol_abs is None else tol_abs, tol if tol_rel is None else tol_rel,
                     max_time, max_iters, max_inner, anderson)


class Problem:
    def __init__(self, path):
        path = os.path.join(path, "")
        self.h = lib().or_load(path.encode())
        if not self.h:
            raise ValueError(lib().or_last_error().decode())
        s = np.zeros(11, dtype=np.int64)
        lib().or_sizes(self.h, s.ctypes.data_as(_lp))
        (self.n, self.nnl, self.ns, self.nx, self.nu, self.ne, self.ydim, self.nulldim,
         self.size_prim, self.size_dual, pre) = [int(v) for v in s]
        self.preconditioned = bool(pre)
        self.size = self.size_prim + self.size_dual
        self.step = lib().or_step_size(self.h)
        self.scaling = np.zeros(self.nx + self.nu)
        lib().or_scaling(self.h, _p(self.scaling))

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_free(self.h)
            self.h = None

    def op(self, prim):
        prim = np.ascontiguousarray(prim, dtype=np.float64)
        out = np.zeros(self.size_dual)
        lib().or_op(self.h, _p(prim), _p(out))
        return out

    def adj(self, dual):
        dual = np.ascontiguousarray(dual, dtype=np.float64)
        out = np.zeros(self.size_prim)
        lib().or_adj(self.h, _p(dual), _p(out))
        return out

    def dot_m(self, x, y):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        return lib().or_dot_m(self.h, _p(x), _p(y))

    def cp_step(self, x0_scaled, z):
        x0 = np.ascontiguousarray(x0_scaled, dtype=np.float64)
        z = np.ascontiguousarray(z, dtype=np.float64)
        out = np.zeros(self.size)
        lib().or_cp_step(self.h, _p(x0), _p(z), _p(out))
        return out

    def project_dynamics(self, x0_scaled, x, u):
        x = np.array(x, dtype=np.float64)
        u = np.array(u, dtype=np.float64)
        x0 = np.ascontiguousarray(x0_scaled, dtype=np.float64)
        lib().or_project_dynamics(self.h, _p(x0), _p(x), _p(u))
        return x, u

    def project_kernel(self, y, t, s):
        y, t, s = (np.array(a, dtype=np.float64) for a in (y, t, s))
        lib().or_project_kernel(self.h, _p(y), _p(t), _p(s))
        return y, t, s

    def project_dual(self, dual):
        d = np.array(dual, dtype=np.float64)
        lib().or_project_dual(self.h, _p(d))
        return d

    def run(self, x0, opts, algo="spock", z=None):
        z0 = np.zeros(self.size) if z is None else np.array(z, dtype=np.float64)
        st = OrStats()
        x0 = np.ascontiguousarray(x0, dtype=np.float64)
        f = lib().or_run_spock if algo == "spock" else lib().or_run_cp
        f(self.h, ctypes.byref(opts), _p(x0), _p(z0), int(z is not None), ctypes.byref(st))
        return z0, st

    def states_inputs(self, z):
        z = np.ascontiguousarray(z, dtype=np.float64)
        xs = np.zeros(self.nx * self.n)
        us = np.zeros(self.nu * self.nnl)
        lib().or_states_inputs(self.h, _p(z), _p(xs), _p(us))
        return xs, us

    def solve_many(self, x0s, opts, threads, keep_z=False):
        x0s = np.ascontiguousarray(x0s, dtype=np.float64).reshape(-1, self.nx)
        cnt = x0s.shape[0]
        status = np.zeros(cnt, dtype=np.int32)
        iters = np.zeros(cnt, dtype=np.int64)
        u0 = np.zeros((cnt, self.nu))
        zs = np.zeros((cnt, self.size)) if keep_z else None
        secs = lib().or_solve_many(self.h, ctypes.byref(opts), cnt, _p(x0s), threads,
                                   status.ctypes.data_as(_ip), iters.ctypes.data_as(_lp), _p(u0),
                                   _p(zs) if keep_z else None)
        return secs, status, iters, u0, zs

    def solve_many_warm(self, x0s, zs, opts, threads, warm=True):
        """Solve each instance, warm-started from its row of zs (count x size) when `warm`; zs
        receives the solutions.  Returns (seconds, status, iters, T calls, u0)."""
        x0s = np.ascontiguousarray(x0s, dtype=np.float64).reshape(-1, self.nx)
        cnt = x0s.shape[0]
        if zs.shape != (cnt, self.size) or zs.dtype != np.float64 or not zs.flags.c_contiguous:
            raise ValueError("zs must be a C-contiguous float64 array of shape (count, size)")
        status = np.zeros(cnt, dtype=np.int32)
        iters = np.zeros(cnt, dtype=np.int64)
        calls = np.zeros(cnt, dtype=np.int64)
        u0 = np.zeros((cnt, self.nu))
        secs = lib().or_solve_many_warm(self.h, ctypes.byref(opts), cnt, _p(x0s), threads,
                                        status.ctypes.data_as(_ip), iters.ctypes.data_as(_lp), _p(u0), _p(zs),
                                        int(warm), calls.ctypes.data_as(_lp))
        return secs, status, iters, calls, u0

    def offline_dynamics(self, AB):
        AB = np.ascontiguousarray(AB, dtype=np.float64)
        n, nnl, nx, nu = self.n, self.nnl, self.nx, self.nu
        P = np.zeros(nx * nx * n)
        K = np.zeros(nu * nx * nnl)
        C = np.zeros(nu * nu * nnl)
        ABK = np.zeros(nx * nx * n)
        APB = np.zeros(nx * nu * n)
        lib().or_offline_dynamics(self.h, _p(AB), _p(P), _p(K), _p(C), _p(ABK), _p(APB))
        return P, K, C, ABK, APB

    def offline_kernel(self, alpha, node):
        out = np.zeros(self.nulldim * self.nulldim)
        lib().or_offline_kernel(self.h, alpha, node, _p(out))
        return out

    def norm_L_sq(self, iters=5000):
        return lib().or_norm_L_sq(self.h, iters)


def project_soc_columns(data, dim):
    d = np.array(data, dtype=np.float64).ravel()
    lib().or_project_soc_columns(_p(d), dim, d.size // dim)
    return d


def project_box(v, lb, ub):
    v = np.array(v, dtype=np.float64)
    lb = np.ascontiguousarray(lb, dtype=np.float64)
    ub = np.ascontiguousarray(ub, dtype=np.float64)
    lib().or_project_box(_p(v), _p(lb), _p(ub), v.size)
    return v
