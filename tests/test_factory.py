"""The product's offline factory (spock_gb300.factory) against the reference factory.

Each golden case under tests/golden/ was written by the reference's Python API
(make_golden.py).  Here the same raw inputs (same random draws) go through this project's
factory, and every tensor it writes must equal the reference's file: tree index arrays,
probabilities, the dynamics cache (problem.py:192-213), AVaR projectors (problem.py:215-231),
cost square roots and translations (build.py:184-668), bounds, scaling and the step size.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, read_bt
from spock_gb300 import factory as F


def build_reftest(path):
    p = np.array([[0.3, 0.7], [0.3, 0.7]])
    tree = F.MarkovChain(p, np.array([0.3, 0.7]), 3, 2).build()
    nx, nu = 3, 2
    dyn = [F.Dynamics(1.5 * np.eye(nx), 1.5 * .5 * np.ones((nx, nu))), F.Dynamics(np.eye(nx), .5 * np.ones((nx, nu)))]
    # tests/cuda/test.py:56-61 scales one shared array in place, so both events end with Q = 2I
    costs = [F.CostQuadratic(2 * np.eye(nx), np.eye(nu)) for _ in range(2)]
    lb = np.concatenate((-np.ones(nx), -5. * np.ones(nu)))
    (F.Factory(tree, nx, nu).with_dynamics_events(dyn).with_cost_nonleaf_events(costs)
     .with_cost_leaf(F.CostQuadratic(3 * np.eye(nx), leaf=True))
     .with_constraint_nonleaf(F.Rectangle(lb, -lb))
     .with_constraint_leaf(F.Rectangle(-.1 * np.ones(nx), .1 * np.ones(nx)))
     .with_risk(F.AVaR(.95)).generate_problem(path))


def build_cfg1(path):
    rng = np.random.default_rng(20261203)
    ne, nx, nu = 3, 3, 2
    P = rng.dirichlet(np.ones(ne), size=ne)
    tree = F.MarkovChain(P, np.ones(ne) / ne, 4, 2).build()
    dyn = [F.Dynamics(np.eye(nx) + .1 * rng.standard_normal((nx, nx)), rng.standard_normal((nx, nu))) for _ in range(ne)]
    Q = np.diag(rng.uniform(1., 10., nx))
    R = np.diag(rng.uniform(.1, 1., nu))
    lb = np.concatenate((-5. * np.ones(nx), -2. * np.ones(nu)))
    (F.Factory(tree, nx, nu).with_dynamics_events(dyn).with_cost_nonleaf(F.CostQuadratic(Q, R))
     .with_cost_leaf(F.CostQuadratic(Q.copy(), leaf=True))
     .with_constraint_nonleaf(F.Rectangle(lb, -lb))
     .with_constraint_leaf(F.Rectangle(-5. * np.ones(nx), 5. * np.ones(nx)))
     .with_risk(F.AVaR(.9)).generate_problem(path))


def build_qpl(path):
    rng = np.random.default_rng(7)
    ne, nx, nu = 3, 4, 2
    tree = F.IidProcess(np.array([.2, .5, .3]), 4, 2).build()
    dyn = []
    for _ in range(ne):
        A = rng.standard_normal((nx, nx)) / np.sqrt(nx)
        A *= 1.05 / max(abs(np.linalg.eigvals(A)))
        dyn.append(F.Dynamics(A, rng.standard_normal((nx, nu))))
    costs = [F.CostQuadraticPlusLinear(np.diag(rng.uniform(1., 10., nx)), rng.standard_normal(nx),
                                       np.diag(rng.uniform(.1, 1., nu)), rng.standard_normal(nu)) for _ in range(ne)]
    leaf = F.CostQuadraticPlusLinear(np.diag(rng.uniform(1., 10., nx)), rng.standard_normal(nx), leaf=True)
    lb = np.concatenate((-3. * np.ones(nx), -1. * np.ones(nu)))
    (F.Factory(tree, nx, nu).with_dynamics_events(dyn).with_cost_nonleaf_events(costs).with_cost_leaf(leaf)
     .with_constraint_nonleaf(F.Rectangle(lb, -lb))
     .with_constraint_leaf(F.Rectangle(-3. * np.ones(nx), 3. * np.ones(nx)))
     .with_risk(F.AVaR(.95)).generate_problem(path))


def build_affpoly(path):
    rng = np.random.default_rng(11)
    ne, nx, nu = 2, 3, 2
    tree = F.MarkovChain(np.array([[.6, .4], [.25, .75]]), np.array([.5, .5]), 3, 2).build()
    dyn = [F.Dynamics(np.eye(nx) + .1 * rng.standard_normal((nx, nx)), rng.standard_normal((nx, nu)),
                      .1 * rng.standard_normal(nx)) for _ in range(ne)]
    costs = [F.CostLinear(rng.standard_normal(nx), rng.standard_normal(nu)) for _ in range(ne)]
    leaf = F.CostLinear(rng.standard_normal(nx), leaf=True)
    G = rng.standard_normal((2, nx + nu))
    poly = F.Polyhedron(G, -np.ones(2), np.ones(2))
    Gl = rng.standard_normal((2, nx))
    (F.Factory(tree, nx, nu).with_dynamics_events(dyn).with_cost_nonleaf_events(costs).with_cost_leaf(leaf)
     .with_constraint_nonleaf(poly).with_constraint_leaf(F.Polyhedron(Gl, -np.ones(2), np.ones(2)))
     .with_risk(F.AVaR(.8)).with_preconditioning(False).generate_problem(path))


BUILDERS = {"reftest": build_reftest, "cfg1": build_cfg1, "qpl": build_qpl, "affpoly": build_affpoly}


@pytest.mark.parametrize("case", sorted(BUILDERS))
def test_factory_matches_reference(case, tmp_path):
    path = str(tmp_path) + "/"
    BUILDERS[case](path)
    ref_dir = os.path.join(GOLDEN, case)
    ref_meta = json.load(open(os.path.join(ref_dir, "data.json")))
    meta = json.load(open(os.path.join(path, "data.json")))
    for k, v in ref_meta.items():
        if k == "stepSize":
            assert abs(meta[k] - v) <= 1e-8 * v
        elif k != "rowsS2":
            assert meta[k] == v, k
    ref_files = sorted(f for f in os.listdir(ref_dir)
                       if f.endswith(".bt") and not f.startswith("test_") and not f.startswith("initialState"))
    assert ref_files == sorted(f for f in os.listdir(path) if f.endswith(".bt"))
    for f in ref_files:
        a, da = read_bt(os.path.join(ref_dir, f))
        b, db = read_bt(os.path.join(path, f))
        assert da == db, f
        if f.endswith("_u.bt"):
            assert np.array_equal(a, b), f
        else:
            # scipy's sqrtm of the root's all-zero cost matrix (never read by the solver) returns
            # non-finite entries; this factory writes zeros there, so compare finite entries only
            fin = np.isfinite(a)
            scale = max(1., np.abs(a[fin]).max()) if fin.any() else 1.
            assert np.allclose(a[fin], b[fin], rtol=0, atol=1e-9 * scale), f


def test_config_sizes(tmp_path):
    """Configuration trees have the node counts of the benchmark definitions."""
    from spock_gb300 import configs
    path, x0 = configs.config1(str(tmp_path / "c1") + "/", seed=3, count=4)
    meta = json.load(open(path + "data.json"))
    assert (meta["numNodes"], meta["numNonleafNodes"], x0.shape) == (31, 22, (4, 3))
    t2 = F.MarkovChain(np.full((3, 3), 1 / 3), np.ones(3) / 3, 10, 4).build()
    assert (t2.num_nodes, t2.num_leaf_nodes) == (607, 81)
    t3 = F.IidProcess(np.ones(5) / 5, 8, 3).build()
    assert (t3.num_nodes, t3.num_leaf_nodes) == (781, 125)


def build_polyid(path, preconditioning=True):
    """Polyhedron-with-identity constraints on nonleaf and leaf nodes (build.py:1025-1096):
    the reference's Python class cannot write fixtures (its assign_dual reads the Gamma block
    from the identity block's offset), so this case is checked against the oracle reading the
    files written here."""
    rng = np.random.default_rng(5)
    ne, nx, nu = 2, 3, 2
    tree = F.MarkovChain(np.array([[.7, .3], [.4, .6]]), np.array([.5, .5]), 3, 2).build()
    dyn = [F.Dynamics(np.eye(nx) + .1 * rng.standard_normal((nx, nx)), rng.standard_normal((nx, nu)))
           for _ in range(ne)]
    Q, R = np.diag(rng.uniform(1., 5., nx)), np.diag(rng.uniform(.1, 1., nu))
    lb = np.concatenate((-4. * np.ones(nx), -2. * np.ones(nu)))
    nl = F.PolyhedronWithIdentity(F.Rectangle(lb, -lb), F.Polyhedron(rng.standard_normal((2, nx + nu)),
                                                                     -np.ones(2), np.ones(2)))
    lf = F.PolyhedronWithIdentity(F.Rectangle(-4. * np.ones(nx), 4. * np.ones(nx)),
                                  F.Polyhedron(rng.standard_normal((3, nx)), -2. * np.ones(3), 2. * np.ones(3)))
    return (F.Factory(tree, nx, nu).with_dynamics_events(dyn).with_cost_nonleaf(F.CostQuadratic(Q, R))
            .with_cost_leaf(F.CostQuadratic(Q.copy(), leaf=True)).with_constraint_nonleaf(nl)
            .with_constraint_leaf(lf).with_risk(F.AVaR(.9)).with_preconditioning(preconditioning)
            .generate_problem(path))


@pytest.mark.parametrize("preconditioning", [False, True])
def test_polyhedron_with_identity(oracle_lib, tmp_path, preconditioning):
    """The factory's L, L* and step size for [I; Gamma] constraints equal the oracle's on the
    written problem; the dual block is the identity rows of every node, then the Gamma rows."""
    path = str(tmp_path) + "/"
    prob = build_polyid(path, preconditioning)
    P = oracle_lib.Problem(path)
    meta = json.load(open(path + "data.json"))
    assert meta["constraint"] == {"nonleaf": "polyhedronWithIdentity", "leaf": "polyhedronWithIdentity"}
    rng = np.random.default_rng(1)
    x, y = rng.standard_normal(P.size_prim), rng.standard_normal(P.size_dual)
    assert np.allclose(prob.op(x), P.op(x), rtol=0, atol=1e-12 * np.abs(P.op(x)).max())
    assert np.allclose(prob.adj(y), P.adj(y), rtol=0, atol=1e-12 * np.abs(P.adj(y)).max())
    assert abs(y @ P.op(x) - P.adj(y) @ x) <= 1e-10 * abs(y @ P.op(x))
    assert abs(.99 / np.sqrt(P.norm_L_sq(20000)) - P.step) <= 1e-8 * P.step
    # identity rows of node 1 hold [x_1; u_1] (scaled); rows after all identity rows hold Gamma
    nnl, nx, nu = prob.tree.num_nonleaf_nodes, 3, 2
    e = np.zeros(P.size_prim)
    e[nu * nnl + nx + 0] = 1.                     # x_1[0]
    d = P.op(e)
    off = prob.y_dim * nnl + nnl                  # after the risk rows and s - b'y
    assert d[off + (nx + nu) * 1 + 0] == 1.
    assert np.count_nonzero(d[off:off + (nx + nu) * nnl]) == 1


def test_config4_mixed(oracle_lib, tmp_path):
    """The mixed batch of config 4: each problem has its own seed and sizes drawn from the given
    ranges, is kept on disk once written, and solves (FP64 oracle, tol 1e-3)."""
    from spock_gb300 import configs
    kw = dict(count=4, nx_range=(3, 6), states_range=(2, 3), horizon_range=(3, 5), stopping_range=(2, 3))
    probs = configs.config4_mixed(str(tmp_path), seed=1, **kw)
    assert len(probs) == 4 and len({p for p, _ in probs}) == 4
    sizes = set()
    for path, x0 in probs:
        meta = json.load(open(path + "data.json"))
        nx, nu = meta["numStates"], meta["numInputs"]
        assert 3 <= nx <= 6 and nu == nx // 2 and x0.shape == (nx,)
        assert 2 <= meta["numEvents"] <= 3 and 4 <= meta["numStages"] <= 6
        sizes.add((nx, meta["numNodes"]))
        P = oracle_lib.Problem(path)
        z, st = P.run(x0, oracle_lib.options(tol=1e-3, anderson=5, max_iters=20000), "spock")
        assert st.status == 0
    assert len(sizes) > 1
    again = configs.config4_mixed(str(tmp_path), seed=1, **kw)
    assert all(a[0] == b[0] and np.array_equal(a[1], b[1]) for a, b in zip(probs, again))
    # written by a pool of two processes: the same files
    par = configs.config4_mixed(str(tmp_path / "pool"), seed=1, workers=2, **kw)
    for (a, xa), (b, xb) in zip(probs, par):
        assert np.array_equal(xa, xb)
        assert open(a + "dynamics_AB_d.bt", "rb").read() == open(b + "dynamics_AB_d.bt", "rb").read()
