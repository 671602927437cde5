"""Offline problem factory: scenario trees, problem data and the offline cache.

This is the offline half of the SPOCK path.  It has the same building blocks and writes the
same files as the reference's Python API (api/python/spock/tree.py, build.py, problem.py):
`data.json` with the keys of api/python/spock/jinja2.py:1-33 and one `.bt` tensor per array
(3 little-endian uint64 dims + column-major payload, `_d` FP64 / `_f` FP32 / `_u` uint64).
The solver library reads those files, so a folder written here and a folder written by the
reference factory are interchangeable.

Everything is numpy FP64.  The offline cache follows the reference's recursions:
  * dynamics projection cache, leaves to root (problem.py:192-213);
  * AVaR nullspace projectors, padded to 4E+1 (problem.py:215-231), computed here as
    I - S'(SS')^-1 S instead of an SVD nullspace basis (same projector);
  * step size 0.99/||L|| with ||L||^2 the largest eigenvalue of L*L (problem.py:402-417);
  * diagonal preconditioning (problem.py:159-190, build.py:70-75, 294-318, 636-668, 914-917).
"""
import json
import os

import numpy as np
import scipy.linalg as sla
from scipy.sparse.linalg import LinearOperator, eigsh

# ------------------------------------------------------------------------------ file I/O


def write_bt(path, arr, dtype):
    """Write a `.bt` tensor: (rows, cols, mats) uint64 header + column-major payload."""
    a = np.asarray(arr)
    if a.ndim == 1:
        a = a.reshape(-1, 1, 1)
    elif a.ndim == 2:
        a = a.reshape(a.shape[0], a.shape[1], 1)
    with open(path, "wb") as fh:
        np.asarray(a.shape, dtype="<u8").tofile(fh)
        np.asarray(a, dtype=dtype).ravel(order="F").tofile(fh)


def read_bt(path):
    with open(path, "rb") as fh:
        dims = np.frombuffer(fh.read(24), dtype="<u8").astype(np.int64)
        kind = path[-4]
        dt = {"d": "<f8", "f": "<f4", "u": "<u8"}[kind]
        a = np.frombuffer(fh.read(), dtype=dt)
    return a.reshape(tuple(dims), order="F")


# ------------------------------------------------------------------------------ trees


class Tree:
    """Scenario tree (tree.py:7-265): nodes numbered stage by stage, children contiguous."""

    def __init__(self, stages, ancestors, probability, events):
        self.stages = np.asarray(stages, dtype=np.int64)
        self.ancestors = np.asarray(ancestors, dtype=np.int64)
        self.probability = np.asarray(probability, dtype=np.float64)
        self.events = np.asarray(events, dtype=np.int64)
        self.num_nodes = len(self.ancestors)
        self.num_stages = int(self.stages[-1]) + 1
        self.num_nonleaf_nodes = int(np.sum(self.stages < self.num_stages - 1))
        self.num_leaf_nodes = self.num_nodes - self.num_nonleaf_nodes
        self.children = [np.flatnonzero(self.ancestors == i) for i in range(self.num_nonleaf_nodes)]
        self.num_children = np.array([len(c) for c in self.children], dtype=np.int64)
        self.num_events = int(self.num_children.max())
        cond = np.empty(self.num_nodes)
        cond[0] = -1.
        cond[1:] = self.probability[1:] / self.probability[self.ancestors[1:]]
        self.cond_prob = cond
        self.stage_from = np.array([np.flatnonzero(self.stages == s)[0] for s in range(self.num_stages)])
        self.stage_to = np.array([np.flatnonzero(self.stages == s)[-1] for s in range(self.num_stages)])

    def write(self, path, dt):
        u = lambda name, v: write_bt(os.path.join(path, name + "_u.bt"), np.asarray(v).astype(np.int64).view(np.uint64), "<u8")
        u("stages", self.stages)
        u("ancestors", self.ancestors)
        u("events", self.events)
        u("childrenFrom", [c[0] for c in self.children])
        u("childrenTo", [c[-1] for c in self.children])
        u("numChildren", self.num_children)
        u("stageFrom", self.stage_from)
        u("stageTo", self.stage_to)
        for name, v in (("probabilities", self.probability), ("conditionalProbabilities", self.cond_prob)):
            write_bt(os.path.join(path, f"{name}_{dt}.bt"), v, _np_dt(dt))


def _np_dt(dt):
    return "<f8" if dt == "d" else "<f4"


def _branching_tree(first, cover_of, horizon, stopping):
    """Node/stage/ancestor layout of tree.py:396-437 (Markov) and 522-559 (i.i.d.)."""
    ancestors = [-1] + [0] * len(first)
    values = [-1] + list(first)
    stages = [0] + [1] * len(first)
    cursor, width = 1, len(first)
    for stage in range(1, stopping):
        added = 0
        new_cursor = cursor + width
        for i in range(width):
            node = cursor + i
            cov = cover_of(values[node])
            ancestors += [node] * len(cov)
            values += list(cov)
            added += len(cov)
        width, cursor = added, new_cursor
        stages += [stage + 1] * added
    for stage in range(stopping, horizon):
        ancestors += list(range(cursor, cursor + width))
        values += values[-width:]
        cursor += width
        stages += [stage + 1] * width
    return np.array(ancestors), np.array(values), np.array(stages)


class MarkovChain:
    """Tree of a stopped Markov chain (tree.py:350-479)."""

    def __init__(self, transition_prob, initial_distribution, horizon, stopping_stage=None):
        self.P = np.asarray(transition_prob, dtype=np.float64)
        self.v = np.asarray(initial_distribution, dtype=np.float64)
        self.N = int(horizon)
        self.tau = int(horizon if stopping_stage is None else stopping_stage)
        if self.tau > self.N:
            raise ValueError("stopping time greater than number of stages")
        for p in list(self.P) + [self.v]:
            if abs(p.sum() - 1) >= 1e-10 or (p < -1e-16).any():
                raise ValueError("invalid probability vector")

    def build(self):
        first = np.flatnonzero(self.v)
        anc, val, stg = _branching_tree(first, lambda w: np.flatnonzero(self.P[w]), self.N, self.tau)
        prob = np.zeros(len(anc))
        prob[0] = 1.
        for i in range(1, len(anc)):
            if stg[i] == 1:
                prob[i] = self.v[val[i]]
            elif stg[i] <= self.tau:
                prob[i] = prob[anc[i]] * self.P[val[anc[i]], val[i]]
            else:
                prob[i] = prob[anc[i]]
        return Tree(stg, anc, prob, val)


class IidProcess:
    """n-ary tree of an i.i.d. process (tree.py:492-588)."""

    def __init__(self, distribution, horizon, stopping_stage=None):
        self.d = np.asarray(distribution, dtype=np.float64).ravel()
        self.N = int(horizon)
        self.tau = int(horizon if stopping_stage is None else stopping_stage)
        if self.tau > self.N:
            raise ValueError("stopping time greater than number of stages")
        if abs(self.d.sum() - 1) >= 1e-10 or (self.d <= 1e-16).any():
            raise ValueError("invalid distribution")

    def build(self):
        cover = np.flatnonzero(self.d)
        anc, val, stg = _branching_tree(cover, lambda w: cover, self.N, self.tau)
        prob = np.zeros(len(anc))
        prob[0] = 1.
        for i in range(1, len(anc)):
            prob[i] = prob[anc[i]] * self.d[val[i]] if stg[i] <= self.tau else prob[anc[i]]
        return Tree(stg, anc, prob, val)


# ------------------------------------------------------------------------------ building blocks


class Dynamics:
    """x+ = A x + B u (+ c) (build.py:13-75)."""

    def __init__(self, A, B, c=None):
        self.A = np.asarray(A, dtype=np.float64)
        self.B = np.asarray(B, dtype=np.float64)
        self.affine = c is not None
        self.c = np.zeros(self.A.shape[0]) if c is None else np.asarray(c, dtype=np.float64).ravel()


class CostQuadratic:
    def __init__(self, Q, R=None, leaf=False):
        self.kind, self.Q, self.R, self.q, self.r, self.leaf = "quadratic", np.asarray(Q, float), R, None, None, leaf
        if R is not None:
            self.R = np.asarray(R, float)


class CostQuadraticPlusLinear:
    def __init__(self, Q, q, R=None, r=None, leaf=False):
        self.kind, self.leaf = "quadraticPlusLinear", leaf
        self.Q, self.q = np.asarray(Q, float), np.asarray(q, float).ravel()
        self.R = None if R is None else np.asarray(R, float)
        self.r = None if r is None else np.asarray(r, float).ravel()


class CostLinear:
    def __init__(self, q, r=None, leaf=False):
        self.kind, self.leaf, self.Q, self.R = "linear", leaf, None, None
        self.q = np.asarray(q, float).ravel()
        self.r = None if r is None else np.asarray(r, float).ravel()


class NoConstraint:
    kind = "no"


class Rectangle:
    kind = "rectangle"

    def __init__(self, lb, ub):
        self.lb, self.ub = np.asarray(lb, float).ravel(), np.asarray(ub, float).ravel()
        if self.lb.size != self.ub.size or (self.lb > self.ub).any():
            raise ValueError("Rectangle constraint bounds invalid")


class RectangleInputBall:
    """Nonleaf constraint (not in the reference): box bounds on the states and the Euclidean ball
    ||u||_2 <= radius on the inputs -- the second-order-cone input constraint ||u||_2 <= r with a
    fixed r.  Its dual block is [x; u] as for a rectangle; the projection clamps the x rows and
    scales u by min(1, r / ||u||)."""
    kind = "rectangleInputBall"

    def __init__(self, x_lb, x_ub, num_inputs, radius):
        x_lb, x_ub = np.asarray(x_lb, float).ravel(), np.asarray(x_ub, float).ravel()
        if x_lb.size != x_ub.size or (x_lb > x_ub).any() or not radius > 0:
            raise ValueError("RectangleInputBall constraint invalid")
        self.lb = np.concatenate((x_lb, -np.inf * np.ones(num_inputs)))
        self.ub = np.concatenate((x_ub, np.inf * np.ones(num_inputs)))
        self.nx = x_lb.size
        self.radius = float(radius)


class Polyhedron:
    kind = "polyhedron"

    def __init__(self, G, lb, ub):
        self.G = np.asarray(G, float)
        self.lb, self.ub = np.asarray(lb, float).ravel(), np.asarray(ub, float).ravel()


class PolyhedronWithIdentity:
    """lb <= [I; Gamma] z <= ub from a Rectangle and a Polyhedron (build.py:1025-1096); the dual
    block holds the identity rows of every node, then the Gamma rows of every node
    (build.py:1050-1070)."""
    kind = "polyhedronWithIdentity"

    def __init__(self, rect, poly):
        if not isinstance(rect, Rectangle) or not isinstance(poly, Polyhedron):
            raise TypeError("PolyhedronWithIdentity takes a Rectangle and a Polyhedron")
        if poly.G.shape[1] != rect.lb.size:
            raise ValueError("PolyhedronWithIdentity: Gamma and the rectangle differ in dimension")
        self.rect, self.poly = rect, poly
        self.lb, self.ub, self.G, self.glb, self.gub = rect.lb, rect.ub, poly.G, poly.lb, poly.ub


class AVaR:
    """AVaR_alpha: E = [alpha I; -I; 1'], b = [p; 0; 1] (build.py:1160-1193)."""
    kind = "avar"

    def __init__(self, alpha):
        if not 0 <= alpha <= 1:
            raise ValueError("AVaR alpha must be in [0, 1]")
        self.alpha = float(alpha)


def _sqrtm(M):
    if np.count_nonzero(M - np.diag(np.diag(M))) == 0:
        return np.diag(np.sqrt(np.maximum(np.diag(M), 0.)))
    return np.real(sla.sqrtm(M))


# ------------------------------------------------------------------------------ problem


class Factory:
    """Same fluent interface as problem.Factory (problem.py:702-879)."""

    def __init__(self, scenario_tree, num_states, num_inputs):
        self.tree, self.nx, self.nu = scenario_tree, int(num_states), int(num_inputs)
        self.dyn_events = None
        self.cost_events = None
        self.leaf_cost = None
        self.nl_con = NoConstraint()
        self.l_con = NoConstraint()
        self.risk = None
        self.precondition = True
        self.cost_scale = 1.

    def with_dynamics(self, d):
        self.dyn_events = [d] * (int(self.tree.events[1:].max()) + 1)
        return self

    def with_dynamics_events(self, ds):
        self.dyn_events = list(ds)
        return self

    def with_cost_nonleaf(self, c):
        self.cost_events = [c] * (int(self.tree.events[1:].max()) + 1)
        return self

    def with_cost_nonleaf_events(self, cs):
        self.cost_events = list(cs)
        return self

    def with_cost_leaf(self, c):
        if not c.leaf:
            raise ValueError("Cannot use nonleaf cost for leaf nodes!")
        self.leaf_cost = c
        return self

    def with_constraint_nonleaf(self, c):
        self.nl_con = c
        return self

    def with_constraint_leaf(self, c):
        self.l_con = c
        return self

    def with_risk(self, r):
        self.risk = r
        return self

    def with_preconditioning(self, enable=True):
        self.precondition = enable
        return self

    def with_cost_scaling(self, factor):
        """Multiply every cost term (Q, R, q, r of the stage and leaf costs) by `factor` > 0.
        Not in the reference factory.  The minimiser (x, u) is unchanged and the optimal value
        is scaled by `factor`; the epigraph variables t, s and the risk variables y shrink with
        it.  Chambolle-Pock takes one step size for the primal and the dual, so a cost-to-go
        orders of magnitude above the state and dual magnitudes slows it down badly (nx = 50,
        Q = diag U[1, 10] gives s_0 near 800); scaling the objective down balances them."""
        if not factor > 0:
            raise ValueError("cost scaling factor must be positive")
        self.cost_scale = float(factor)
        return self

    def generate_problem(self, path, dt="d", step_size=None, offline="host", device=0):
        """Write the problem to `path`.  offline="host" computes the offline cache here in numpy
        (dynamics cache, nullspace projectors, ARPACK step size); offline="gpu" writes the
        problem data only and has the library compute the cache on GPU `device` in FP64
        (`spock_offline_complete`), as the C++ generator does."""
        if offline not in ("host", "gpu"):
            raise ValueError("offline must be 'host' or 'gpu'")
        f = self
        if self.cost_scale != 1.:
            import copy
            f = copy.copy(self)
            f.cost_events = [_scale_cost(c, self.cost_scale) for c in self.cost_events]
            f.leaf_cost = _scale_cost(self.leaf_cost, self.cost_scale)
            f.cost_scale = 1.
        return Problem(f, path, dt, step_size, gpu_device=device if offline == "gpu" else None)


def _scale_cost(cost, factor):
    import copy
    c = copy.copy(cost)
    for name in ("Q", "R", "q", "r"):
        v = getattr(c, name, None)
        if v is not None:
            setattr(c, name, factor * np.asarray(v, float))
    return c


class Problem:
    """Problem data + offline cache, written to `path` (problem.py:16-687)."""

    def __init__(self, f, path, dt="d", step_size=None, gpu_device=None):
        t, nx, nu = f.tree, f.nx, f.nu
        self.tree, self.nx, self.nu = t, nx, nu
        n, nnl = t.num_nodes, t.num_nonleaf_nodes
        ev = t.events
        # per-node dynamics (node 0 carries zeros, problem.py:744-757)
        A = np.zeros((n, nx, nx))
        B = np.zeros((n, nx, nu))
        c = np.zeros((n, nx))
        for i in range(1, n):
            d = f.dyn_events[ev[i]]
            A[i], B[i], c[i] = d.A, d.B, d.c
        self.affine = f.dyn_events[0].affine
        cost_kind = f.cost_events[0].kind
        leaf = f.leaf_cost
        Q = np.zeros((n, nx, nx))
        R = np.zeros((n, nu, nu))
        q = np.zeros((n, nx))
        r = np.zeros((n, nu))
        for i in range(1, n):
            ce = f.cost_events[ev[i]]
            if ce.Q is not None:
                Q[i] = ce.Q
            if ce.R is not None:
                R[i] = ce.R
            if ce.q is not None:
                q[i] = ce.q
            if ce.r is not None:
                r[i] = ce.r
        lQ = np.zeros((nx, nx)) if leaf.Q is None else leaf.Q.copy()
        lq = np.zeros(nx) if leaf.q is None else leaf.q.copy()
        # preconditioning (problem.py:159-190)
        self.preconditioned = False
        sx, su = np.ones(nx), np.ones(nu)
        if f.precondition:
            for k in range(nx):
                cand = [sx[k]]
                if cost_kind != "linear":
                    cand += list(np.sqrt(Q[1:, k, k]))
                if cost_kind != "quadratic":
                    cand += list(np.abs(q[1:, k]))
                if leaf.kind != "linear":
                    cand.append(np.sqrt(lQ[k, k]))
                if leaf.kind != "quadratic":
                    cand.append(abs(lq[k]))
                sx[k] = max(cand)
            for k in range(nu):
                cand = [su[k]]
                if cost_kind != "linear":
                    cand += list(np.sqrt(R[1:, k, k]))
                if cost_kind != "quadratic":
                    cand += list(np.abs(r[1:, k]))
                su[k] = max(cand)
            mul = np.sqrt(t.num_children.max())
            sx, su = sx * mul, su * mul
            self.preconditioned = not (np.allclose(sx, 1.) and np.allclose(su, 1.))
        if not self.preconditioned:
            sx, su = np.ones(nx), np.ones(nu)
        self.scaling = np.concatenate((sx, su))
        Sx, Sxi, Sui = np.diag(sx), np.diag(1 / sx), np.diag(1 / su)
        if self.preconditioned:
            A[1:] = Sx @ A[1:] @ Sxi
            B[1:] = Sx @ B[1:] @ Sui
            c[1:] = c[1:] * sx
            Q[1:] = Sxi @ Q[1:] @ Sxi
            R[1:] = Sui @ R[1:] @ Sui
            q[1:] = q[1:] / sx
            r[1:] = r[1:] / su
            lQ = Sxi @ lQ @ Sxi
            lq = lq / sx
        self.A, self.B, self.c = A, B, c
        self.cost_kind, self.leaf_kind = cost_kind, leaf.kind
        # cost data (build.py:184-668)
        if cost_kind != "linear":
            cache = {}
            sQ = np.zeros_like(Q)
            sR = np.zeros_like(R)
            for i in range(1, n):
                key = ev[i]
                if key not in cache:
                    cache[key] = (_sqrtm(Q[i]), _sqrtm(R[i]))
                sQ[i], sR[i] = cache[key]
            trans = np.zeros((n, nx + nu + 2))
            for i in range(1, n):
                if cost_kind == "quadratic":
                    trans[i, -2:] = (-.5, .5)
                else:
                    a = .5 * np.linalg.solve(sQ[i], q[i])
                    b = .5 * np.linalg.solve(sR[i], r[i])
                    nq = -.125 * q[i] @ np.linalg.solve(Q[i], q[i]) - .125 * r[i] @ np.linalg.solve(R[i], r[i])
                    trans[i] = np.concatenate((a, b, [-.5 + nq, .5 + nq]))
            self.sqrtQ, self.sqrtR, self.trans = sQ, sR, trans
        self.q, self.r = q, r
        if leaf.kind != "linear":
            self.lsqrtQ = _sqrtm(lQ)
            if leaf.kind == "quadratic":
                self.ltrans = np.concatenate((np.zeros(nx), [-.5, .5]))
            else:
                a = .5 * np.linalg.solve(self.lsqrtQ, lq)
                nq = -.125 * lq @ np.linalg.solve(lQ, lq)
                self.ltrans = np.concatenate((a, [-.5 + nq, .5 + nq]))
        self.lq = lq
        # constraints (constraints.cuh bounds; build.py:914-917, 1016-1019 conditioning)
        self.nl_con, self.l_con = f.nl_con, f.l_con
        scale_xu = self.scaling
        self.nl_bounds = self._con_data(f.nl_con, scale_xu)
        self.l_bounds = self._con_data(f.l_con, sx)
        # risk (build.py:1184-1193) and kernel projectors (problem.py:215-231, 263-267)
        E = t.num_events
        self.alpha = f.risk.alpha
        self.null_dim = 4 * E + 1
        self.y_dim = 2 * E + 1
        self.b = np.zeros((nnl, self.y_dim))
        for i in range(nnl):
            ch = t.children[i]
            m = len(ch)
            self.b[i, :m] = t.cond_prob[ch]
            self.b[i, 2 * m] = 1.
        self._sizes()
        self.path = path
        if gpu_device is not None:
            self._write(path, dt, with_cache=False)
            from . import offline_complete
            gpu_step = offline_complete(path, gpu_device)
            self.step_size = float(step_size) if step_size is not None else gpu_step
            if step_size is not None:
                self._write_step_size(path)
            self._read_cache(path, dt)
            return
        self.nntr = np.zeros((nnl, self.null_dim, self.null_dim))
        for i in range(nnl):
            m = len(t.children[i])
            S = np.zeros((m, self.null_dim))
            S[np.arange(m), np.arange(m)] = self.alpha
            S[np.arange(m), m + np.arange(m)] = -1.
            S[:, 2 * m] = 1.
            S[np.arange(m), self.y_dim + np.arange(m)] = -1.
            S[np.arange(m), self.y_dim + E + np.arange(m)] = -1.
            self.nntr[i] = np.eye(self.null_dim) - S.T @ np.linalg.solve(S @ S.T, S)
        self._offline_dynamics()
        self.step_size = float(step_size) if step_size is not None else self._step_size()
        self._write(path, dt)

    def _read_cache(self, path, dt):
        """The offline cache as the GPU wrote it, in this object's (mats, rows, cols) layout."""
        get = lambda name: np.transpose(read_bt(os.path.join(path, name + "_" + dt + ".bt")), (2, 0, 1))
        self.P, self.K, self.lowChol = get("dynamics_P"), get("dynamics_K"), get("dynamics_lowCholesky")
        self.ABKTr, self.APB, self.nntr = get("dynamics_ABKTr"), get("dynamics_APB"), get("risk_NNtr")

    def _write_step_size(self, path):
        fn = os.path.join(path, "data.json")
        meta = json.load(open(fn))
        meta["stepSize"] = float(self.step_size)
        with open(fn, "w") as fh:
            json.dump(meta, fh, indent=1)

    @staticmethod
    def _con_data(con, scale):
        if con.kind == "no":
            return None
        if con.kind == "rectangle":
            return (con.lb * scale, con.ub * scale)
        if con.kind == "rectangleInputBall":
            su = scale[con.nx:]
            if not np.allclose(su, su[0]):
                raise ValueError("an input ball needs the same preconditioning scale on every input "
                                 "(or with_preconditioning(False))")
            return (con.lb * scale, con.ub * scale, con.radius * su[0])
        if con.kind == "polyhedron":
            return (con.G / scale[None, :], con.lb, con.ub)
        if con.kind == "polyhedronWithIdentity":
            return (con.G / scale[None, :], con.glb, con.gub, con.lb * scale, con.ub * scale)
        raise ValueError("constraint kind %s not supported by this factory" % con.kind)

    def _offline_dynamics(self):
        """problem.py:192-213 (leaves to root)."""
        t, nx, nu = self.tree, self.nx, self.nu
        n, nnl = t.num_nodes, t.num_nonleaf_nodes
        P = np.zeros((n, nx, nx))
        P[nnl:] = np.eye(nx)
        K = np.zeros((nnl, nu, nx))
        L = np.zeros((nnl, nu, nu))
        ABKTr = np.zeros((n, nx, nx))
        APB = np.zeros((n, nx, nu))
        A, B = self.A, self.B
        for i in reversed(range(nnl)):
            ch = t.children[i]
            BtP = np.transpose(B[ch], (0, 2, 1)) @ P[ch]
            Rt = np.eye(nu) + (BtP @ B[ch]).sum(0)
            sk = (BtP @ A[ch]).sum(0)
            L[i] = np.linalg.cholesky(Rt)
            K[i] = sla.cho_solve((L[i], True), -sk)
            Abk = A[ch] + B[ch] @ K[i]
            AbkT = np.transpose(Abk, (0, 2, 1))
            ABKTr[ch] = AbkT
            APB[ch] = AbkT @ P[ch] @ B[ch]
            P[i] = np.eye(nx) + K[i].T @ K[i] + (AbkT @ P[ch] @ Abk).sum(0)
        self.P, self.K, self.lowChol, self.ABKTr, self.APB = P, K, L, ABKTr, APB

    def _sizes(self):
        t, nx, nu = self.tree, self.nx, self.nu
        n, nnl, nl = t.num_nodes, t.num_nonleaf_nodes, t.num_leaf_nodes
        self.size_prim = (nu + self.y_dim) * nnl + (nx + 2) * n
        d3 = {"no": 0, "rectangle": nx + nu, "rectangleInputBall": nx + nu}.get(self.nl_con.kind, None)
        d3 = self.nl_bounds[0].shape[0] + (nx + nu if self.nl_con.kind == "polyhedronWithIdentity" else 0) \
            if d3 is None else d3
        d5 = {"no": 0, "rectangle": nx}.get(self.l_con.kind, None)
        d5 = self.l_bounds[0].shape[0] + (nx if self.l_con.kind == "polyhedronWithIdentity" else 0) \
            if d5 is None else d5
        d4 = 2 if self.cost_kind == "linear" else nx + nu + 2
        d6 = 2 if self.leaf_kind == "linear" else nx + 2
        self.size_dual = self.y_dim * nnl + nnl + d3 * nnl + d4 * n + d5 * nl + d6 * nl

    # -- vectorised L and L* (problem.py:273-365), used for the step size
    def _split_prim(self, p):
        t, nx, nu, yd = self.tree, self.nx, self.nu, self.y_dim
        n, nnl = t.num_nodes, t.num_nonleaf_nodes
        o = 0
        u = p[o:o + nu * nnl].reshape(nnl, nu); o += nu * nnl
        x = p[o:o + nx * n].reshape(n, nx); o += nx * n
        y = p[o:o + yd * nnl].reshape(nnl, yd); o += yd * nnl
        tt = p[o:o + n]; o += n
        s = p[o:o + n]
        return u, x, y, tt, s

    def op(self, p):
        t, nx, nu = self.tree, self.nx, self.nu
        n, nnl = t.num_nodes, t.num_nonleaf_nodes
        u, x, y, tt, s = self._split_prim(p)
        out = [y.ravel(), s[:nnl] - np.einsum("ij,ij->i", self.b, y)]
        xu = np.concatenate((x[:nnl], u), axis=1)
        if self.nl_con.kind in ("rectangle", "rectangleInputBall"):
            out.append(xu.ravel())
        elif self.nl_con.kind == "polyhedron":
            out.append((xu @ self.nl_bounds[0].T).ravel())
        elif self.nl_con.kind == "polyhedronWithIdentity":
            out += [xu.ravel(), (xu @ self.nl_bounds[0].T).ravel()]
        anc = t.ancestors[1:]
        xa, ua = x[anc], u[anc]
        if self.cost_kind == "linear":
            s4 = np.zeros(n)
            s4[1:] = np.einsum("ij,ij->i", self.q[1:], xa) + np.einsum("ij,ij->i", self.r[1:], ua)
            out += [s4, tt]
        else:
            iv = np.zeros((n, nx + nu + 2))
            iv[1:, :nx] = np.einsum("nij,nj->ni", self.sqrtQ[1:], xa)
            iv[1:, nx:nx + nu] = np.einsum("nij,nj->ni", self.sqrtR[1:], ua)
            h = .5 * tt[1:]
            if self.cost_kind == "quadraticPlusLinear":
                h = h - .5 * (np.einsum("ij,ij->i", self.q[1:], xa) + np.einsum("ij,ij->i", self.r[1:], ua))
            iv[1:, -2] = h
            iv[1:, -1] = h
            out.append(iv.ravel())
        xl, sl = x[nnl:], s[nnl:]
        if self.l_con.kind == "rectangle":
            out.append(xl.ravel())
        elif self.l_con.kind == "polyhedron":
            out.append((xl @ self.l_bounds[0].T).ravel())
        elif self.l_con.kind == "polyhedronWithIdentity":
            out += [xl.ravel(), (xl @ self.l_bounds[0].T).ravel()]
        if self.leaf_kind == "linear":
            out += [xl @ self.lq, sl]
        else:
            vi = np.zeros((len(sl), nx + 2))
            vi[:, :nx] = xl @ self.lsqrtQ.T
            h = .5 * sl - (.5 * (xl @ self.lq) if self.leaf_kind == "quadraticPlusLinear" else 0.)
            vi[:, -2] = h
            vi[:, -1] = h
            out.append(vi.ravel())
        return np.concatenate(out)

    def adj(self, d):
        t, nx, nu, yd = self.tree, self.nx, self.nu, self.y_dim
        n, nnl, nl = t.num_nodes, t.num_nonleaf_nodes, t.num_leaf_nodes
        o = 0
        I = d[o:o + yd * nnl].reshape(nnl, yd); o += yd * nnl
        II = d[o:o + nnl]; o += nnl
        x = np.zeros((n, nx))
        u = np.zeros((nnl, nu))
        tt = np.zeros(n)
        s = np.zeros(n)
        s[:nnl] = II
        y = I - self.b * II[:, None]
        if self.nl_con.kind in ("rectangle", "rectangleInputBall"):
            III = d[o:o + (nx + nu) * nnl].reshape(nnl, nx + nu); o += (nx + nu) * nnl
            x[:nnl] = III[:, :nx]
            u[:] = III[:, nx:]
        elif self.nl_con.kind == "polyhedron":
            G = self.nl_bounds[0]
            III = d[o:o + G.shape[0] * nnl].reshape(nnl, G.shape[0]); o += G.shape[0] * nnl
            xu = III @ G
            x[:nnl] = xu[:, :nx]
            u[:] = xu[:, nx:]
        elif self.nl_con.kind == "polyhedronWithIdentity":
            G = self.nl_bounds[0]
            xu = d[o:o + (nx + nu) * nnl].reshape(nnl, nx + nu).copy(); o += (nx + nu) * nnl
            xu += d[o:o + G.shape[0] * nnl].reshape(nnl, G.shape[0]) @ G; o += G.shape[0] * nnl
            x[:nnl] = xu[:, :nx]
            u[:] = xu[:, nx:]
        anc = t.ancestors[1:]
        if self.cost_kind == "linear":
            s4 = d[o:o + n]; o += n
            tt[:] = d[o:o + n]; o += n
            np.add.at(x, anc, self.q[1:] * s4[1:, None])
            np.add.at(u, anc, self.r[1:] * s4[1:, None])
        else:
            iv = d[o:o + (nx + nu + 2) * n].reshape(n, nx + nu + 2); o += (nx + nu + 2) * n
            d23 = iv[1:, -2] + iv[1:, -1]
            cx = np.einsum("nij,nj->ni", self.sqrtQ[1:], iv[1:, :nx])
            cu = np.einsum("nij,nj->ni", self.sqrtR[1:], iv[1:, nx:nx + nu])
            if self.cost_kind == "quadraticPlusLinear":
                cx = cx - .5 * self.q[1:] * d23[:, None]
                cu = cu - .5 * self.r[1:] * d23[:, None]
            np.add.at(x, anc, cx)
            np.add.at(u, anc, cu)
            tt[1:] = .5 * d23
        if self.l_con.kind == "rectangle":
            x[nnl:] = d[o:o + nx * nl].reshape(nl, nx); o += nx * nl
        elif self.l_con.kind == "polyhedron":
            G = self.l_bounds[0]
            x[nnl:] = d[o:o + G.shape[0] * nl].reshape(nl, G.shape[0]) @ G; o += G.shape[0] * nl
        elif self.l_con.kind == "polyhedronWithIdentity":
            G = self.l_bounds[0]
            x[nnl:] = d[o:o + nx * nl].reshape(nl, nx); o += nx * nl
            x[nnl:] += d[o:o + G.shape[0] * nl].reshape(nl, G.shape[0]) @ G; o += G.shape[0] * nl
        if self.leaf_kind == "linear":
            x[nnl:] += d[o:o + nl, None] * self.lq[None, :]; o += nl
            s[nnl:] = d[o:o + nl]
        else:
            vi = d[o:o + (nx + 2) * nl].reshape(nl, nx + 2)
            d23 = vi[:, -2] + vi[:, -1]
            x[nnl:] += vi[:, :nx] @ self.lsqrtQ.T
            if self.leaf_kind == "quadraticPlusLinear":
                x[nnl:] -= .5 * d23[:, None] * self.lq[None, :]
            s[nnl:] = .5 * d23
        return np.concatenate((u.ravel(), x.ravel(), y.ravel(), tt, s))

    def _step_size(self):
        op = LinearOperator((self.size_prim, self.size_prim), matvec=lambda v: self.adj(self.op(v)),
                            dtype=np.float64)
        lam = eigsh(op, k=1, which="LA", tol=1e-10, v0=np.ones(self.size_prim))[0][0]
        return .99 / np.sqrt(lam)

    # -- files
    def _write(self, path, dt, with_cache=True):
        """The folder; with_cache=False leaves out the offline cache and writes stepSize 0 (the
        input of spock_offline_complete)."""
        os.makedirs(path, exist_ok=True)
        t, nx, nu = self.tree, self.nx, self.nu
        fdt = _np_dt(dt)
        t.write(path, dt)
        ext = "_" + dt + ".bt"
        w = lambda name, arr: write_bt(os.path.join(path, name + ext), arr, fdt)
        stack = lambda a: np.transpose(a, (1, 2, 0))  # (mats, r, c) -> (r, c, mats)
        AB = np.concatenate((self.A, self.B), axis=2)
        w("dynamics_BTr", stack(np.transpose(self.B, (0, 2, 1))))
        w("dynamics_AB", stack(AB))
        if with_cache:
            w("dynamics_P", stack(self.P))
            w("dynamics_K", stack(self.K))
            w("dynamics_ABKTr", stack(self.ABKTr))
            w("dynamics_APB", stack(self.APB))
            w("dynamics_lowCholesky", stack(self.lowChol))
        if self.affine:
            w("dynamics_c", stack(self.c[:, :, None]))
        if with_cache:
            w("risk_NNtr", stack(self.nntr))
        w("risk_b", stack(self.b[:, :, None]))
        if self.preconditioned:
            w("scaling", self.scaling)
        n = t.num_nodes
        if self.cost_kind == "linear":
            w("nonleafCost_gradient", stack(np.concatenate((self.q, self.r), axis=1)[:, None, :]))
        else:
            w("nonleafCost_sqrtQ", stack(self.sqrtQ))
            w("nonleafCost_sqrtR", stack(self.sqrtR))
            w("nonleafCost_translation", stack(self.trans[:, :, None]))
            if self.cost_kind == "quadraticPlusLinear":
                w("nonleafCost_q", stack(self.q[:, :, None]))
                w("nonleafCost_r", stack(self.r[:, :, None]))
        if self.leaf_kind == "linear":
            w("leafCost_gradient", self.lq[None, :, None])
        else:
            w("leafCost_sqrtQ", self.lsqrtQ[:, :, None])
            w("leafCost_translation", self.ltrans)
            if self.leaf_kind == "quadraticPlusLinear":
                w("leafCost_q", self.lq)
        for txt, con, bnd in (("nonleafConstraint", self.nl_con, self.nl_bounds),
                              ("leafConstraint", self.l_con, self.l_bounds)):
            if con.kind in ("rectangle", "rectangleInputBall"):
                w(txt + "ILB", bnd[0])
                w(txt + "IUB", bnd[1])
                if con.kind == "rectangleInputBall":
                    w(txt + "Radius", np.array([bnd[2]]))
            elif con.kind in ("polyhedron", "polyhedronWithIdentity"):
                w(txt + "Gamma", bnd[0])
                w(txt + "GLB", bnd[1])
                w(txt + "GUB", bnd[2])
                if con.kind == "polyhedronWithIdentity":
                    w(txt + "ILB", bnd[3])
                    w(txt + "IUB", bnd[4])
        meta = {
            "numEvents": int(t.num_events), "numNonleafNodes": int(t.num_nonleaf_nodes),
            "numNodes": int(n), "numStages": int(t.num_stages), "numStates": nx, "numInputs": nu,
            "dynamics": {"type": "affine" if self.affine else "linear"},
            "cost": {"nonleaf": self.cost_kind, "leaf": self.leaf_kind},
            "constraint": {"nonleaf": self.nl_con.kind, "leaf": self.l_con.kind},
            "risk": {"type": "avar", "alpha": self.alpha},
            "rowsS2": int(t.num_events), "rowsNNtr": int(self.null_dim),
            "stepSize": float(self.step_size) if with_cache else 0.,
            "preconditioned": bool(self.preconditioned),
        }
        with open(os.path.join(path, "data.json"), "w") as fh:
            json.dump(meta, fh, indent=1)
