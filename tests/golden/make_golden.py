"""Generate the golden fixtures under tests/golden/ with the reference's own Python factory.

The reference SPOCK package (api/python/spock in ruairimoran/spock.cu) builds the scenario
tree, the problem data and the offline cache, and writes them as `data.json` plus `.bt`
tensors.  With `with_tests()` it also writes operator fixtures: a random primal, `L` of it,
`L*` of that, an adjoint identity and an M-inner-product (problem.py:367-435, 586-604).

Two of its imports are absent from this environment and are stubbed here:

* `gputils_api.write_array_to_gputils_binary_file` -- the `.bt` writer.  The format is the
  one the reference's Julia reader documents (tests/julia/modelFactory/src/modelFactory.jl:26-60):
  three little-endian uint64 (rows, cols, mats) followed by the column-major payload.
* `turtle` -- only used by the tree plot (tree.py:267-347).

`Problem.__test_dynamic_programming` needs cvxpy (absent); it is replaced by a no-op that
leaves the DP fixtures empty.

Run from the repository root (it needs the reference checkout, so it runs only where that
exists):  python tests/golden/make_golden.py /path/to/reference
"""
import os
import shutil
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _bt_write(arr, path):
    a = np.asarray(arr)
    if a.ndim == 1:
        shape = (a.shape[0], 1, 1)
    elif a.ndim == 2:
        shape = (a.shape[0], a.shape[1], 1)
    elif a.ndim == 3:
        shape = a.shape
    else:
        raise ValueError("bad rank")
    a3 = a.reshape(shape, order="F") if a.ndim < 3 else a
    with open(path, "wb") as fh:
        np.asarray(shape, dtype="<u8").tofile(fh)
        # column-major within each matrix, matrices stacked along the 3rd axis
        np.asfortranarray(a3).ravel(order="F").astype(a.dtype.newbyteorder("<")).tofile(fh)


def _install_stubs():
    ga = types.ModuleType("gputils_api")
    ga.write_array_to_gputils_binary_file = _bt_write
    sys.modules["gputils_api"] = ga
    sys.modules["turtle"] = types.ModuleType("turtle")


def _import_reference(ref_root):
    sys.dont_write_bytecode = True
    _install_stubs()
    sys.path.insert(0, os.path.join(ref_root, "api", "python"))
    import spock  # noqa: E402
    prob_cls = spock.problem.Problem

    def _no_dp(self):
        self._Problem__dp_test_states = np.zeros(0)
        self._Problem__dp_test_inputs = np.zeros(0)
        self._Problem__dp_projected_states = np.zeros(0)
        self._Problem__dp_projected_inputs = np.zeros(0)

    prob_cls._Problem__test_dynamic_programming = _no_dp
    return spock


def case_reftest(s):
    """The reference's own CUDA-test problem (tests/cuda/test.py:15-98), FP64."""
    p = np.array([[0.3, 0.7], [0.3, 0.7]])
    v = np.array([0.3, 0.7])
    tree = s.tree.MarkovChain(transition_prob=p, initial_distribution=v, horizon=3,
                              stopping_stage=2, dt='d').build()
    nx, nu = 3, 2
    A = np.eye(nx)
    B = 0.5 * np.ones((nx, nu))
    dynamics = [s.build.Dynamics(1.5 * A, 1.5 * B), s.build.Dynamics(A, B)]
    q = np.eye(nx)
    r = np.eye(nu)
    nonleaf_costs = []
    for i in range(1, 3):
        q *= i
        nonleaf_costs += [s.build.CostQuadratic(q, r)]
    leaf_cost = s.build.CostQuadratic(3 * np.eye(nx), leaf=True)
    si_lb = np.vstack((-1. * np.ones((nx, 1)), -5. * np.ones((nu, 1))))
    si_ub = -si_lb
    nonleaf_constraint = s.build.Rectangle(si_lb, si_ub)
    leaf_constraint = s.build.Rectangle(-.1 * np.ones((nx, 1)), .1 * np.ones((nx, 1)))
    (s.problem.Factory(scenario_tree=tree, num_states=nx, num_inputs=nu)
     .with_dynamics_events(dynamics)
     .with_cost_nonleaf_events(nonleaf_costs)
     .with_cost_leaf(leaf_cost)
     .with_constraint_nonleaf(nonleaf_constraint)
     .with_constraint_leaf(leaf_constraint)
     .with_risk(s.build.AVaR(.95))
     .with_preconditioning()
     .with_tests()
     .generate_problem())


def case_cfg1(s):
    """Small random RAOCP: 3-state Markov chain (Dirichlet rows), N=4, tau=2, nx=3, nu=2,
    Q=diag U[1,10], R=diag U[0.1,1], Qf=Q, AVaR(0.9), box |x|<=5, |u|<=2.  Seeded."""
    rng = np.random.default_rng(20261203)
    ne, nx, nu = 3, 3, 2
    P = rng.dirichlet(np.ones(ne), size=ne)
    v = np.ones(ne) / ne
    tree = s.tree.MarkovChain(transition_prob=P, initial_distribution=v, horizon=4,
                              stopping_stage=2, dt='d').build()
    dyn = [s.build.Dynamics(np.eye(nx) + .1 * rng.standard_normal((nx, nx)),
                            rng.standard_normal((nx, nu))) for _ in range(ne)]
    Q = np.diag(rng.uniform(1., 10., nx))
    R = np.diag(rng.uniform(.1, 1., nu))
    lb = np.concatenate((-5. * np.ones(nx), -2. * np.ones(nu)))
    (s.problem.Factory(scenario_tree=tree, num_states=nx, num_inputs=nu)
     .with_dynamics_events(dyn)
     .with_cost_nonleaf(s.build.CostQuadratic(Q, R))
     .with_cost_leaf(s.build.CostQuadratic(Q.copy(), leaf=True))
     .with_constraint_nonleaf(s.build.Rectangle(lb, -lb))
     .with_constraint_leaf(s.build.Rectangle(-5. * np.ones(nx), 5. * np.ones(nx)))
     .with_risk(s.build.AVaR(.9))
     .with_tests()
     .generate_problem())
    x0 = rng.uniform(-1., 1., nx)
    tree.write_to_file_fp("initialState", x0)


def case_qpl(s):
    """Quadratic-plus-linear costs, i.i.d. tree with 3 events, N=4, tau=2, nx=4, nu=2.
    Exercises the q/r translations (build.py:522-535) and the linear epigraph terms."""
    rng = np.random.default_rng(7)
    ne, nx, nu = 3, 4, 2
    tree = s.tree.IidProcess(distribution=np.array([.2, .5, .3]), horizon=4,
                             stopping_stage=2, dt='d').build()
    dyn = []
    for _ in range(ne):
        A = rng.standard_normal((nx, nx)) / np.sqrt(nx)
        A *= 1.05 / max(abs(np.linalg.eigvals(A)))
        dyn.append(s.build.Dynamics(A, rng.standard_normal((nx, nu))))
    costs = [s.build.CostQuadraticPlusLinear(np.diag(rng.uniform(1., 10., nx)), rng.standard_normal(nx),
                                             np.diag(rng.uniform(.1, 1., nu)), rng.standard_normal(nu))
             for _ in range(ne)]
    leaf = s.build.CostQuadraticPlusLinear(np.diag(rng.uniform(1., 10., nx)), rng.standard_normal(nx),
                                           leaf=True)
    lb = np.concatenate((-3. * np.ones(nx), -1. * np.ones(nu)))
    (s.problem.Factory(scenario_tree=tree, num_states=nx, num_inputs=nu)
     .with_dynamics_events(dyn)
     .with_cost_nonleaf_events(costs)
     .with_cost_leaf(leaf)
     .with_constraint_nonleaf(s.build.Rectangle(lb, -lb))
     .with_constraint_leaf(s.build.Rectangle(-3. * np.ones(nx), 3. * np.ones(nx)))
     .with_risk(s.build.AVaR(.95))
     .with_tests()
     .generate_problem())
    x0 = rng.uniform(-1., 1., nx)
    tree.write_to_file_fp("initialState", x0)


def case_affpoly(s):
    """Affine dynamics, linear costs and polyhedral constraints, Markov 2 states, N=3, tau=2,
    nx=3, nu=2, no preconditioning.  (The reference's Python `PolyhedronWithIdentity` fails its
    own adjoint self-test -- its `assign_dual` reads the Gamma block from the identity block's
    offset, build.py:1060-1066 -- so it cannot produce fixtures.)"""
    rng = np.random.default_rng(11)
    ne, nx, nu = 2, 3, 2
    P = np.array([[.6, .4], [.25, .75]])
    tree = s.tree.MarkovChain(transition_prob=P, initial_distribution=np.array([.5, .5]), horizon=3,
                              stopping_stage=2, dt='d').build()
    dyn = [s.build.Dynamics(np.eye(nx) + .1 * rng.standard_normal((nx, nx)), rng.standard_normal((nx, nu)),
                            .1 * rng.standard_normal(nx)) for _ in range(ne)]
    costs = [s.build.CostLinear(rng.standard_normal(nx), rng.standard_normal(nu)) for _ in range(ne)]
    leaf = s.build.CostLinear(rng.standard_normal(nx), leaf=True)
    G = rng.standard_normal((2, nx + nu))
    poly = s.build.Polyhedron(G, -np.ones(2), np.ones(2))
    Gl = rng.standard_normal((2, nx))
    (s.problem.Factory(scenario_tree=tree, num_states=nx, num_inputs=nu)
     .with_dynamics_events(dyn)
     .with_cost_nonleaf_events(costs)
     .with_cost_leaf(leaf)
     .with_constraint_nonleaf(poly)
     .with_constraint_leaf(s.build.Polyhedron(Gl, -np.ones(2), np.ones(2)))
     .with_risk(s.build.AVaR(.8))
     .with_preconditioning(False)
     .with_tests()
     .generate_problem())


CASES = {"reftest": case_reftest, "cfg1": case_cfg1, "qpl": case_qpl, "affpoly": case_affpoly}


def main(ref_root):
    s = _import_reference(ref_root)
    for name, fn in CASES.items():
        np.random.seed(1234)  # the factory draws its test fixtures from np.random
        work = tempfile.mkdtemp()
        cwd = os.getcwd()
        os.chdir(work)
        try:
            fn(s)
        finally:
            os.chdir(cwd)
        out = os.path.join(HERE, name)
        if os.path.isdir(out):
            shutil.rmtree(out)
        shutil.copytree(os.path.join(work, "data"), out)
        shutil.rmtree(work)
        print("wrote", out, len(os.listdir(out)), "files")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference checkout>")
    main(sys.argv[1])
