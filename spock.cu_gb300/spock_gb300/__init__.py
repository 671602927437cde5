"""GB300-native SPOCK solver: Python host interface over the C ABI (include/spock_gb300.h).

The classes mirror the reference's C++ interface (ruairimoran/spock.cu, src/tree.cuh,
src/problem.cuh, src/cache.cuh):

    tree = ScenarioTree("path/to/data/")
    data = ProblemData(tree)
    cache = CacheBuilder(tree, data).tol(1e-4).maxIters(2000).andersonBuffer(5).build()
    status = cache.runSpock(x0)            # 0 converged, 1 out of iterations, 2 out of time
    u, x = cache.inputs(), cache.states()

with two additions for the GB300 path: `.precision(32|64)` and `.batch(B)` on the builder,
and `Cache.runSpockBatch(x0s)` to solve B instances (different initial states, same tree and
problem data) in one device-resident loop.  Errors raise ValueError (the reference throws
std::invalid_argument) or RuntimeError for CUDA failures.  There is no CPU fallback: the
compiled library must be present (`build()`), and a missing library raises at import time of
the first call.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG, "_build", "libspock_gb300.so")

CONVERGED, OUT_OF_ITER, OUT_OF_TIME, DIVERGED, NOT_RUN = 0, 1, 2, 3, -1
_STATUS_TEXT = {NOT_RUN: "Cache has not been run!", CONVERGED: "Converged!", OUT_OF_ITER: "Out of iterations!",
                OUT_OF_TIME: "Out of time!", DIVERGED: "Stopped on a non-finite residual."}


def toString(status):
    """Status text (cache.cuh:75-88)."""
    return _STATUS_TEXT.get(status, "Unknown status.")


class Options(ctypes.Structure):
    _fields_ = [("tol_abs", ctypes.c_double), ("tol_rel", ctypes.c_double), ("max_time_secs", ctypes.c_double),
                ("max_iters", ctypes.c_long), ("max_inner", ctypes.c_long), ("anderson", ctypes.c_long),
                ("precision", ctypes.c_int), ("batch", ctypes.c_long), ("device", ctypes.c_int)]


_dp = ctypes.POINTER(ctypes.c_double)
_lp = ctypes.POINTER(ctypes.c_long)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p

_SIGS = {
    "spock_options_default": (None, [ctypes.POINTER(Options)]),
    "spock_last_error": (ctypes.c_char_p, []),
    "spock_problem_load": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_vp)]),
    "spock_problem_free": (None, [_vp]),
    "spock_problem_sizes": (ctypes.c_int, [_vp, _lp]),
    "spock_problem_step": (ctypes.c_int, [_vp, _dp, _dp]),
    "spock_solver_create": (ctypes.c_int, [_vp, ctypes.POINTER(Options), ctypes.POINTER(_vp)]),
    "spock_solver_free": (None, [_vp]),
    "spock_solve": (ctypes.c_int, [_vp, ctypes.c_int, _dp, ctypes.c_long, _dp, _ip, _lp]),
    "spock_solve_device": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _ip, _lp]),
    "spock_get_iterate": (ctypes.c_int, [_vp, ctypes.c_long, _dp]),
    "spock_get_iterates": (ctypes.c_int, [_vp, _dp]),
    "spock_get_states_inputs": (ctypes.c_int, [_vp, ctypes.c_long, _dp, _dp]),
    "spock_get_first_inputs": (ctypes.c_int, [_vp, _dp]),
    "spock_status": (ctypes.c_int, [_vp, ctypes.c_long, _ip, _lp, _dp]),
    "spock_counters": (ctypes.c_int, [_vp, _lp]),
    "spock_reset": (ctypes.c_int, [_vp]),
    "spock_op": (ctypes.c_int, [_vp, _dp, _dp]),
    "spock_adj": (ctypes.c_int, [_vp, _dp, _dp]),
    "spock_cp_step": (ctypes.c_int, [_vp, _dp, _dp, _dp]),
    "spock_apply_m": (ctypes.c_int, [_vp, _dp, _dp]),
    "spock_kernel_time": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_int, _dp, _lp]),
    "spock_round_time": (ctypes.c_int, [_vp, ctypes.c_int, _dp]),
    "spock_run_stats": (ctypes.c_int, [_vp, _lp, _lp, _lp]),
    "spock_tuning": (ctypes.c_int, [_vp, _ip]),
    "spock_counters_all": (ctypes.c_int, [_vp, _lp]),
    "spock_set_tuning": (ctypes.c_int, [_vp, _ip]),
    "spock_set_fp64_finish": (ctypes.c_int, [_vp, ctypes.c_long]),
    "spock_step_size": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp]),
    "spock_copy_iterate": (ctypes.c_int, [_vp, _vp]),
    "spock_solve_group": (ctypes.c_int, [ctypes.c_long, ctypes.POINTER(_vp), ctypes.c_int, ctypes.POINTER(_dp), _lp,
                                         ctypes.POINTER(_ip), ctypes.POINTER(_lp)]),
    "spock_set_iterate_device": (ctypes.c_int, [_vp, _vp, ctypes.c_int]),
    "spock_mlp_create": (ctypes.c_int, [_ip, ctypes.c_int, ctypes.POINTER(_vp)]),
    "spock_mlp_free": (None, [_vp]),
    "spock_mlp_param_count": (ctypes.c_long, [_vp]),
    "spock_mlp_set_params": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_float)]),
    "spock_mlp_get_params": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    "spock_mlp_forward": (ctypes.c_int, [_vp, _vp, ctypes.c_int, _vp]),
    "spock_mlp_train_step": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, ctypes.c_float, ctypes.POINTER(ctypes.c_float)]),
    "spock_offline_dynamics": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _dp, _dp]),
    "spock_offline_complete": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, _dp]),
    "spock_resolve": (ctypes.c_int, [_vp, ctypes.c_int, _dp, ctypes.c_long, _ip, _lp]),
    "spock_resolve_device": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _ip, _lp]),
    "spock_project_dynamics_noalloc": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "spock_get_dual": (ctypes.c_int, [_vp, _dp, _dp]),
    "spock_reduce_check": (ctypes.c_int, [_vp, _dp, _dp, _dp]),
    "spock_gemm_bf16": (ctypes.c_int, [_vp, _vp, ctypes.c_long, ctypes.c_long, ctypes.c_int, ctypes.c_float, _vp, _vp,
                                       ctypes.c_int, _vp, _vp, ctypes.c_long, ctypes.c_int]),
    "spock_warm_start_pca": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, _vp]),
}

_lib = None


def build():
    """Compile the CUDA library in-tree (nvcc, sm_103a)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_spock_build", os.path.join(PKG, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build()


def lib():
    """The loaded C-ABI library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libspock_gb300.so not built ({LIB_PATH}); run spock_gb300.build()")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(rc):
    if rc == 0:
        return
    msg = lib().spock_last_error().decode()
    if rc == 1:
        raise ValueError(msg)
    raise RuntimeError(msg)


def _p(a):
    return a.ctypes.data_as(_dp)


def offline_complete(path, device=0, iters=20000):
    """Write the offline cache of a data folder whose problem data is written: the dynamics cache,
    the AVaR nullspace projectors and the step size, computed on GPU `device` in FP64
    (problem.py:192-231, 402-417).  Returns the step size."""
    step = ctypes.c_double()
    _check(lib().spock_offline_complete(os.path.join(path, "").encode(), int(device), int(iters), ctypes.byref(step)))
    return step.value


class ScenarioTree:
    """Scenario tree read from a data folder (tree.cuh:102-179).  The folder also carries the
    problem data, which ProblemData reads (in the reference they are two passes over the
    same files)."""

    def __init__(self, path="./data/"):
        self._path = os.path.join(path, "")
        h = _vp()
        _check(lib().spock_problem_load(self._path.encode(), ctypes.byref(h)))
        self._h = h
        s = np.zeros(10, dtype=np.int64)
        _check(lib().spock_problem_sizes(h, s.ctypes.data_as(_lp)))
        (self._ne, self._n, self._nnl, self._ns, self._nx, self._nu, self._sp, self._sd, pre, self._nd) = [int(v) for v in s]
        self._pre = bool(pre)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().spock_problem_free(self._h)
            self._h = None

    def path(self): return self._path

    def offlineDynamics(self, device=0, replace=False):
        """The dynamics projection's offline cache (problem.py:192-213) recomputed on the GPU in
        FP64 from this problem's [A B]: dict of P, K, lowChol, ABKTr, APB in the .bt layouts.
        With replace=True solvers created afterwards use it."""
        n, nnl, nx, nu = self._n, self._nnl, self._nx, self._nu
        out = {"P": np.zeros(nx * nx * n), "K": np.zeros(nu * nx * nnl), "lowChol": np.zeros(nu * nu * nnl),
               "ABKTr": np.zeros(nx * nx * n), "APB": np.zeros(nx * nu * n)}
        _check(lib().spock_offline_dynamics(self._h, device, int(replace), _p(out["P"]), _p(out["K"]),
                                            _p(out["lowChol"]), _p(out["ABKTr"]), _p(out["APB"])))
        return out

    def numEvents(self): return self._ne
    def numNodes(self): return self._n
    def numNonleafNodes(self): return self._nnl
    def numLeafNodes(self): return self._n - self._nnl
    def numStages(self): return self._ns
    def numStates(self): return self._nx
    def numInputs(self): return self._nu


class ProblemData:
    """Problem data of a tree's folder (problem.cuh:126-153)."""

    def __init__(self, tree):
        self._tree = tree
        step = ctypes.c_double()
        self._scaling = np.zeros(tree.numStates() + tree.numInputs())
        _check(lib().spock_problem_step(tree._h, ctypes.byref(step), _p(self._scaling)))
        self._step = step.value

    def stepSize(self): return self._step
    def stepSizeRecip(self): return 1. / self._step
    def preconditioned(self): return self._tree._pre
    def scaling(self): return self._scaling.copy()
    def nullDim(self): return self._tree._nd
    def yDim(self): return self._tree._nd - 2 * self._tree._ne


class CacheBuilder:
    """Fluent solver builder with the reference defaults (cache.cuh:1138-1245)."""

    def __init__(self, tree, data):
        self._tree, self._data = tree, data
        o = Options()
        lib().spock_options_default(ctypes.byref(o))
        self._o = o
        self._debug = False

    def toleranceAbsolute(self, tol): self._o.tol_abs = tol; return self
    def toleranceRelative(self, tol): self._o.tol_rel = tol; return self

    def tol(self, tol):
        self._o.tol_abs = tol
        self._o.tol_rel = tol
        return self

    def maxTimeSecs(self, t): self._o.max_time_secs = t; return self
    def maxIters(self, n): self._o.max_iters = int(n); return self
    def maxItersInner(self, n): self._o.max_inner = int(n); return self
    def andersonBuffer(self, m): self._o.anderson = int(m); return self

    def enableDebug(self, enable=True):
        if enable and self._o.max_iters == 0:
            self._o.max_iters = 1000
        self._debug = enable
        return self

    # GB300 additions
    def precision(self, bits): self._o.precision = int(bits); return self
    def batch(self, b): self._o.batch = int(b); return self
    def device(self, d): self._o.device = int(d); return self

    def build(self):
        return Cache(self._tree, self._data, self._o)

    make_unique = build


class Cache:
    """SPOCK solver (cache.cuh:94-430).  Iterates are kept on the device between calls."""

    def __init__(self, tree, data, opts):
        self._tree, self._data = tree, data
        self._B = int(opts.batch)
        self._dtype = np.float64 if opts.precision == 64 else np.float32
        h = _vp()
        _check(lib().spock_solver_create(tree._h, ctypes.byref(opts), ctypes.byref(h)))
        self._h = h
        self._status = np.full(self._B, NOT_RUN, dtype=np.int32)
        self._iters = np.zeros(self._B, dtype=np.int64)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().spock_solver_free(self._h)
            self._h = None

    def sizePrimal(self): return self._tree._sp
    def sizeDual(self): return self._tree._sd
    def sizeIterate(self): return self._tree._sp + self._tree._sd
    def batchSize(self): return self._B

    def _run(self, algo, x0, prev):
        x0 = np.ascontiguousarray(np.atleast_2d(np.asarray(x0, dtype=np.float64)))
        if x0.shape[1] != self._tree.numStates():
            raise ValueError(f"[initialiseState] Error initialising state: problem setup for "
                             f"{self._tree.numStates()} but given {x0.shape[1]} states")
        warm = None
        if prev is not None:
            warm = np.ascontiguousarray(np.asarray(prev, dtype=np.float64).reshape(-1, self.sizeIterate()))
            if warm.shape[0] != x0.shape[0]:
                raise ValueError("one previous iterate per initial state is required")
        _check(lib().spock_solve(self._h, algo, _p(x0), x0.shape[0], _p(warm) if warm is not None else None,
                                 self._status.ctypes.data_as(_ip), self._iters.ctypes.data_as(_lp)))
        return int(self._status[0])

    def runSpock(self, x0, prev=None):
        """SuperMann-accelerated CP from initial state x0 (cache.cuh:1008-1132); `prev` is a
        previous full iterate to warm start from."""
        return self._run(0, x0, prev)

    def runCp(self, x0, prev=None):
        """Plain Chambolle-Pock (cache.cuh:967-1002)."""
        return self._run(1, x0, prev)

    def runSpockBatch(self, x0s, prev=None):
        """Solve every instance of the batch; x0s has one row per instance (rows are reused
        cyclically when fewer than the batch).  Returns the status array."""
        self._run(0, x0s, prev)
        return self._status.copy()

    def runCpBatch(self, x0s, prev=None):
        self._run(1, x0s, prev)
        return self._status.copy()

    def resolveBatch(self, x0s, algo=0):
        """Re-solve every instance warm-started from the current iterate (the previous solve's
        solution, on the device) with new initial states.  Returns the status array."""
        x0 = np.ascontiguousarray(np.atleast_2d(np.asarray(x0s, dtype=np.float64)))
        if x0.shape[1] != self._tree.numStates():
            raise ValueError("[initialiseState] wrong number of states")
        _check(lib().spock_resolve(self._h, algo, _p(x0), x0.shape[0], self._status.ctypes.data_as(_ip),
                                   self._iters.ctypes.data_as(_lp)))
        return self._status.copy()

    def resolveDevice(self, x0_device_ptr, algo=0):
        """resolveBatch with the initial states on the device (as solveDevice)."""
        _check(lib().spock_resolve_device(self._h, algo, ctypes.c_void_p(x0_device_ptr),
                                          self._status.ctypes.data_as(_ip), self._iters.ctypes.data_as(_lp)))
        return self._status.copy()

    def setIterateDevice(self, z_device_ptr, bits):
        """Take the iterate from a device array (sizeIterate x batch, element-major, FP32 or FP64)."""
        _check(lib().spock_set_iterate_device(self._h, ctypes.c_void_p(z_device_ptr), int(bits)))

    def copyIterateFrom(self, other):
        """Take another solver's current iterate (same problem and batch, same GPU), converted to
        this solver's precision on the device."""
        _check(lib().spock_copy_iterate(self._h, other._h))

    def polish(self, fp32_solver, x0s):
        """FP64 polish: continue from `fp32_solver`'s solution under this (FP64) solver's
        tolerances, with the same initial states.  Returns the status array."""
        self.copyIterateFrom(fp32_solver)
        return self.resolveBatch(x0s)

    def status(self, instance=0): return int(self._status[instance])
    def statuses(self): return self._status.copy()
    def solveIter(self, instance=0): return int(self._iters[instance])
    def solveIters(self): return self._iters.copy()

    def solveTime(self):
        t = ctypes.c_double()
        _check(lib().spock_status(self._h, 0, None, None, ctypes.byref(t)))
        return t.value

    def solution(self, instance=0):
        out = np.zeros(self.sizeIterate())
        _check(lib().spock_get_iterate(self._h, instance, _p(out)))
        return out

    def solutions(self):
        out = np.zeros((self._B, self.sizeIterate()))
        _check(lib().spock_get_iterates(self._h, _p(out)))
        return out

    def solutionPrim(self, instance=0): return self.solution(instance)[:self.sizePrimal()]
    def solutionDual(self, instance=0): return self.solution(instance)[self.sizePrimal():]

    def states(self, instance=0):
        xs = np.zeros(self._tree.numStates() * self._tree.numNodes())
        _check(lib().spock_get_states_inputs(self._h, instance, _p(xs), None))
        return xs

    def inputs(self, instance=0):
        us = np.zeros(self._tree.numInputs() * self._tree.numNonleafNodes())
        _check(lib().spock_get_states_inputs(self._h, instance, None, _p(us)))
        return us

    def firstInputs(self):
        out = np.zeros((self._B, self._tree.numInputs()))
        _check(lib().spock_get_first_inputs(self._h, _p(out)))
        return out

    def counters(self):
        out = np.zeros(7, dtype=np.int64)
        _check(lib().spock_counters(self._h, out.ctypes.data_as(_lp)))
        return dict(zip(["K0", "K1", "K2", "bt", "K3", "calls_T", "iters"], out.tolist()))

    def countersAll(self):
        """Per-instance counters, a (batch, 7) array: K0, K1, K2, backtracks, K3, T calls, iterations."""
        out = np.zeros((self._B, 7), dtype=np.int64)
        _check(lib().spock_counters_all(self._h, out.ctypes.data_as(_lp)))
        return out

    def reset(self):
        _check(lib().spock_reset(self._h))
        self._status[:] = NOT_RUN

    # operator-level access (what the reference tests reach through friend declarations)
    def op(self, prim):
        prim = np.ascontiguousarray(prim, dtype=np.float64)
        out = np.zeros(self.sizeDual())
        _check(lib().spock_op(self._h, _p(prim), _p(out)))
        return out

    def adj(self, dual):
        dual = np.ascontiguousarray(dual, dtype=np.float64)
        out = np.zeros(self.sizePrimal())
        _check(lib().spock_adj(self._h, _p(dual), _p(out)))
        return out

    def cpStep(self, x0, z):
        x0 = np.ascontiguousarray(x0, dtype=np.float64)
        z = np.ascontiguousarray(z, dtype=np.float64)
        out = np.zeros(self.sizeIterate())
        _check(lib().spock_cp_step(self._h, _p(x0), _p(z), _p(out)))
        return out

    def getDual(self, primal):
        """Cache::getDual (cache.cuh:371-376): the dual candidate for the primal candidate
        `primal` at the current iterate."""
        primal = np.ascontiguousarray(primal, dtype=np.float64)
        if primal.shape != (self.sizePrimal(),):
            raise ValueError("[getDual] primal has the wrong size")
        out = np.zeros(self.sizeDual())
        _check(lib().spock_get_dual(self._h, _p(primal), _p(out)))
        return out

    def applyM(self, z):
        z = np.ascontiguousarray(z, dtype=np.float64)
        out = np.zeros(self.sizeIterate())
        _check(lib().spock_apply_m(self._h, _p(z), _p(out)))
        return out

    def dotM(self, x, y):
        """x' M y (cache.cuh:721-734)."""
        return float(np.dot(np.asarray(x, dtype=np.float64), self.applyM(y)))

    def kernelTime(self, which, reps=20):
        ms = ctypes.c_double()
        b = ctypes.c_long()
        _check(lib().spock_kernel_time(self._h, which.encode(), reps, ctypes.byref(ms), ctypes.byref(b)))
        return ms.value, b.value

    def tuning(self):
        """Tile shapes chosen by the autotuner for L*, L and the dynamics sweep (runs it if needed)."""
        out = np.zeros(5, dtype=np.int32)
        _check(lib().spock_tuning(self._h, out.ctypes.data_as(_ip)))
        return dict(zip(["lstar_tiles_per_cta", "lstar_double_buffer", "lop_tiles_per_cta", "lop_double_buffer",
                         "dyn_tiles_per_cta"], out.tolist()))

    def stepSize(self, iters=5000):
        """(||L||^2, 0.99 / ||L||) by the power iteration on the GPU (problem.py:402-417)."""
        lam, step = ctypes.c_double(), ctypes.c_double()
        _check(lib().spock_step_size(self._h, int(iters), ctypes.byref(lam), ctypes.byref(step)))
        return lam.value, step.value

    def fp64Finish(self, rounds):
        """FP32 batched solvers: after `rounds` rounds, the last <= 32 running instances continue
        the same iteration in FP64 (spock_set_fp64_finish); 0 turns it off."""
        _check(lib().spock_set_fp64_finish(self._h, int(rounds)))
        return self

    def setTuning(self, lstar, lop, dyn):
        """Override the autotuner's tiles per CTA (1, 2, 4 or 8) for L*, L and the dynamics sweep."""
        v = np.array([lstar, lop, dyn], dtype=np.int32)
        _check(lib().spock_set_tuning(self._h, v.ctypes.data_as(_ip)))

    def runStats(self):
        """(rounds, kernel launches) of the last solve."""
        r, l = ctypes.c_long(), ctypes.c_long()
        _check(lib().spock_run_stats(self._h, ctypes.byref(r), ctypes.byref(l), None))
        return r.value, l.value

    def compactions(self):
        """Instance compactions of the last solve."""
        c = ctypes.c_long()
        _check(lib().spock_run_stats(self._h, None, None, ctypes.byref(c)))
        return c.value

    def solveDevice(self, x0_device_ptr, algo=0):
        """Solve with initial states already on the device (nx x batch, element-major, in the
        solver precision).  Returns the status array."""
        _check(lib().spock_solve_device(self._h, algo, ctypes.c_void_p(x0_device_ptr),
                                        self._status.ctypes.data_as(_ip), self._iters.ctypes.data_as(_lp)))
        return self._status.copy()

    def roundTime(self, rounds=20):
        ms = ctypes.c_double()
        _check(lib().spock_round_time(self._h, rounds, ctypes.byref(ms)))
        return ms.value


def solve_group(caches, x0s, algo=0):
    """Mixed batch: cold-start solves of several solvers (different problems) at once, one host
    thread and CUDA stream each.  x0s[i] has rows for caches[i].  Returns the status arrays."""
    n = len(caches)
    if n != len(x0s):
        raise ValueError("one x0 array per solver")
    xs = [np.ascontiguousarray(np.atleast_2d(np.asarray(x, dtype=np.float64))) for x in x0s]
    for c, x in zip(caches, xs):
        if x.shape[1] != c._tree.numStates():
            raise ValueError("[initialiseState] wrong number of states")
    hs = (_vp * n)(*[c._h for c in caches])
    xp = (_dp * n)(*[_p(x) for x in xs])
    cnt = np.array([x.shape[0] for x in xs], dtype=np.int64)
    sp = (_ip * n)(*[c._status.ctypes.data_as(_ip) for c in caches])
    ip = (_lp * n)(*[c._iters.ctypes.data_as(_lp) for c in caches])
    _check(lib().spock_solve_group(n, hs, algo, xp, cnt.ctypes.data_as(_lp), sp, ip))
    return [c._status.copy() for c in caches]
