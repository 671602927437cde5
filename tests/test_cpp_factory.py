"""The C++ problem generator (include/spock_gb300_factory.hpp) and the GPU offline cache
(spock_offline_complete) against the Python factory, which is itself pinned to folders written
by the reference factory (test_factory.py).

The same raw inputs go to both: Python draws them, writes them as `.bt` tensors with a spec
file, and tests/cpp/factory_main.cpp builds the problem from them.  On the CPU the C++ folder
without its offline cache must hold exactly the Python folder's other files with the same
contents; on the GPU the completed folder (dynamics cache, AVaR nullspace projectors, step size
computed in FP64 on the device) must match the Python factory's numpy/ARPACK cache.
"""
import json
import os
import subprocess
import time

import numpy as np
import pytest

from conftest import ROOT, read_bt
import spock_gb300 as sg
from spock_gb300 import factory as F

CACHE = ("dynamics_P", "dynamics_K", "dynamics_lowCholesky", "dynamics_ABKTr", "dynamics_APB", "risk_NNtr")


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    lib = sg.build()
    out = str(tmp_path_factory.mktemp("cppfactory") / "factory_main")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "factory_main.cpp"), "-o", out,
                           "-L", os.path.dirname(lib), "-lspock_gb300", "-Wl,-rpath," + os.path.dirname(lib)])
    return out


def _spd(rng, n, diagonal):
    if diagonal:
        return np.diag(rng.uniform(1., 10., n))
    M = rng.standard_normal((n, n))
    return M @ M.T / n + np.eye(n)


def make_case(name, nx=None, nu=None):
    """Raw inputs of one test problem: (spec dict, arrays dict)."""
    rng = np.random.default_rng({"cfg1": 1, "qpl_affine_poly": 2, "linear_ball": 3, "cfg2": 4}[name])
    if name == "cfg1":
        ne, nx, nu = 3, 3, 2
        spec = dict(tree="markov", horizon=4, stopping=2, nx=nx, nu=nu, events=ne, dynamics="linear",
                    cost="quadratic", leaf="quadratic", nlcon="rectangle", lcon="rectangle", alpha=.9,
                    precondition=1, scale=1., dtype="d")
        arr = dict(tree_P=rng.dirichlet(np.ones(ne), size=ne), tree_v=np.ones(ne) / ne)
        diag = True
    elif name == "cfg2":
        ne, nx, nu = 3, nx or 50, nu or 20
        spec = dict(tree="markov", horizon=10, stopping=4, nx=nx, nu=nu, events=ne, dynamics="linear",
                    cost="quadraticPlusLinear", leaf="quadraticPlusLinear", nlcon="rectangle", lcon="rectangle",
                    alpha=.95, precondition=1, scale=1e-3, dtype="d")
        arr = dict(tree_P=rng.dirichlet(np.ones(ne), size=ne), tree_v=np.ones(ne) / ne)
        diag = True
    elif name == "qpl_affine_poly":
        ne, nx, nu = 3, 4, 2
        spec = dict(tree="iid", horizon=4, stopping=2, nx=nx, nu=nu, events=ne, dynamics="affine",
                    cost="quadraticPlusLinear", leaf="quadraticPlusLinear", nlcon="polyhedronWithIdentity",
                    lcon="polyhedron", alpha=.7, precondition=1, scale=.5, dtype="d")
        arr = dict(tree_d=np.array([.2, .5, .3]))
        diag = False
    else:  # linear_ball: a Markov chain with a zero transition and a zero initial probability
        ne, nx, nu = 2, 3, 3
        spec = dict(tree="markov", horizon=5, stopping=3, nx=nx, nu=nu, events=ne, dynamics="linear",
                    cost="linear", leaf="linear", nlcon="rectangleInputBall", lcon="no", alpha=1.,
                    precondition=0, scale=1., dtype="f", radius=1.5)
        arr = dict(tree_P=np.array([[.6, .4], [0., 1.]]), tree_v=np.array([1., 0.]))
        diag = True
    A = np.empty((ne, nx, nx))
    for e in range(ne):
        A[e] = rng.standard_normal((nx, nx)) / np.sqrt(nx)
        A[e] *= 1.05 / max(abs(np.linalg.eigvals(A[e])))
    arr.update(dyn_A=A, dyn_B=rng.standard_normal((ne, nx, nu)), dyn_c=rng.standard_normal((ne, nx, 1)),
               cost_Q=np.array([_spd(rng, nx, diag) for _ in range(ne)]),
               cost_R=np.array([.1 * _spd(rng, nu, diag) for _ in range(ne)]),
               cost_q=rng.standard_normal((ne, nx, 1)), cost_r=rng.standard_normal((ne, nu, 1)),
               leaf_Q=_spd(rng, nx, diag)[None], leaf_q=rng.standard_normal(nx))
    xu = nx + nu
    if spec["nlcon"] in ("rectangle", "polyhedronWithIdentity"):
        arr.update(nl_lb=-rng.uniform(1., 3., xu), nl_ub=rng.uniform(1., 3., xu))
    if spec["nlcon"] == "rectangleInputBall":
        arr.update(nl_lb=-3. * np.ones(nx), nl_ub=3. * np.ones(nx))
    if spec["nlcon"] == "polyhedronWithIdentity":
        arr.update(nl_G=rng.standard_normal((2, xu)), nl_glb=-np.ones(2), nl_gub=np.ones(2))
    if spec["lcon"] == "rectangle":
        arr.update(l_lb=-rng.uniform(1., 3., nx), l_ub=rng.uniform(1., 3., nx))
    if spec["lcon"] == "polyhedron":
        arr.update(l_G=rng.standard_normal((3, nx)), l_glb=-np.ones(3), l_gub=2. * np.ones(3))
    return spec, arr


def write_inputs(d, spec, arr):
    os.makedirs(d, exist_ok=True)
    with open(os.path.join(d, "spec.txt"), "w") as fh:
        for k, v in spec.items():
            fh.write(f"{k} {v!r}\n" if isinstance(v, float) else f"{k} {v}\n")
    for k, v in arr.items():
        v = np.asarray(v, float)
        if k.startswith(("dyn_", "cost_")) or k == "leaf_Q":
            v = np.transpose(v, (1, 2, 0))  # (events, r, c) -> (r, c, events)
        F.write_bt(os.path.join(d, k + "_d.bt"), v, "<f8")


def python_factory(spec, arr, path, offline="host"):
    """The same problem through spock_gb300.factory."""
    ne = spec["events"]
    tree = (F.MarkovChain(arr["tree_P"], arr["tree_v"], spec["horizon"], spec["stopping"]) if spec["tree"] == "markov"
            else F.IidProcess(arr["tree_d"], spec["horizon"], spec["stopping"])).build()
    affine = spec["dynamics"] == "affine"
    dyn = [F.Dynamics(arr["dyn_A"][e], arr["dyn_B"][e], arr["dyn_c"][e, :, 0] if affine else None) for e in range(ne)]
    ck, lk = spec["cost"], spec["leaf"]
    Q, R, q, r = arr["cost_Q"], arr["cost_R"], arr["cost_q"][:, :, 0], arr["cost_r"][:, :, 0]
    if ck == "quadratic":
        costs = [F.CostQuadratic(Q[e], R[e]) for e in range(ne)]
    elif ck == "quadraticPlusLinear":
        costs = [F.CostQuadraticPlusLinear(Q[e], q[e], R[e], r[e]) for e in range(ne)]
    else:
        costs = [F.CostLinear(q[e], r[e]) for e in range(ne)]
    lQ, lq = arr["leaf_Q"][0], arr["leaf_q"]
    leaf = {"quadratic": lambda: F.CostQuadratic(lQ, leaf=True),
            "quadraticPlusLinear": lambda: F.CostQuadraticPlusLinear(lQ, lq, leaf=True),
            "linear": lambda: F.CostLinear(lq, leaf=True)}[lk]()

    def con(kind, p):
        if kind == "no":
            return F.NoConstraint()
        if kind == "rectangle":
            return F.Rectangle(arr[p + "lb"], arr[p + "ub"])
        if kind == "polyhedron":
            return F.Polyhedron(arr[p + "G"], arr[p + "glb"], arr[p + "gub"])
        if kind == "polyhedronWithIdentity":
            return F.PolyhedronWithIdentity(F.Rectangle(arr[p + "lb"], arr[p + "ub"]),
                                            F.Polyhedron(arr[p + "G"], arr[p + "glb"], arr[p + "gub"]))
        return F.RectangleInputBall(arr[p + "lb"], arr[p + "ub"], spec["nu"], spec["radius"])

    return (F.Factory(tree, spec["nx"], spec["nu"]).with_dynamics_events(dyn).with_cost_nonleaf_events(costs)
            .with_cost_leaf(leaf).with_constraint_nonleaf(con(spec["nlcon"], "nl_"))
            .with_constraint_leaf(con(spec["lcon"], "l_")).with_risk(F.AVaR(spec["alpha"]))
            .with_preconditioning(bool(spec["precondition"])).with_cost_scaling(spec["scale"])
            .generate_problem(path, dt=spec["dtype"], offline=offline))


def compare_folders(mine, ref, with_cache, rtol, cache_rtol=1e-9):
    """Every tensor and data.json key of `ref` against `mine` (the cache only with_cache)."""
    ref_files = sorted(f for f in os.listdir(ref) if f.endswith(".bt"))
    mine_files = sorted(f for f in os.listdir(mine) if f.endswith(".bt"))
    expect = ref_files if with_cache else [f for f in ref_files if not f.rsplit("_", 1)[0] in CACHE]
    assert mine_files == expect
    for f in expect:
        (a, da), (b, db) = read_bt(os.path.join(mine, f)), read_bt(os.path.join(ref, f))
        assert da == db, f
        if f.endswith("_u.bt"):
            assert np.array_equal(a, b), f
            continue
        tol = cache_rtol if f.rsplit("_", 1)[0] in CACHE else rtol
        a, b = np.asarray(a, float), np.asarray(b, float)
        fin = np.isfinite(b)
        assert np.array_equal(np.isfinite(a), fin) and np.array_equal(a[~fin], b[~fin]), f
        scale = max(1., np.abs(b[fin]).max()) if fin.any() else 1.
        assert np.abs(a[fin] - b[fin]).max(initial=0.) <= tol * scale, f
    ja, jb = json.load(open(os.path.join(mine, "data.json"))), json.load(open(os.path.join(ref, "data.json")))
    step_a, step_b = ja.pop("stepSize"), jb.pop("stepSize")
    assert ja == jb
    return step_a, step_b


CASES = ["cfg1", "qpl_affine_poly", "linear_ball"]


@pytest.mark.parametrize("case", CASES)
def test_cpp_problem_data_matches_python_factory(exe, tmp_path, case):
    spec, arr = make_case(case)
    write_inputs(str(tmp_path / "in"), spec, arr)
    python_factory(spec, arr, str(tmp_path / "py") + "/")
    r = subprocess.run([exe, "data", str(tmp_path / "in"), str(tmp_path / "cpp")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rtol = 1e-6 if spec["dtype"] == "f" else 1e-11
    step_cpp, _ = compare_folders(str(tmp_path / "cpp"), str(tmp_path / "py"), False, rtol)
    assert step_cpp == 0.


@pytest.mark.parametrize("case", ["markov", "iid", "stopping", "horizon", "alpha", "rectangle", "leafcost"])
def test_cpp_factory_rejects_invalid_input(exe, case):
    r = subprocess.run([exe, "bad", case], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("invalid_argument"), r.stdout + r.stderr


def test_folder_without_cache_is_not_a_problem(exe, tmp_path):
    """A folder written without its offline cache (stepSize 0) is refused by the loader until
    the cache is computed."""
    spec, arr = make_case("cfg1")
    write_inputs(str(tmp_path / "in"), spec, arr)
    assert subprocess.run([exe, "data", str(tmp_path / "in"), str(tmp_path / "cpp")]).returncode == 0
    with pytest.raises(ValueError):
        sg.ScenarioTree(str(tmp_path / "cpp"))


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_cpp_generator_with_gpu_offline_cache(exe, tmp_path, case):
    """The complete C++ folder: problem data on the host, dynamics cache, nullspace projectors and
    step size on the GPU in FP64, against the numpy/ARPACK factory."""
    spec, arr = make_case(case)
    write_inputs(str(tmp_path / "in"), spec, arr)
    python_factory(spec, arr, str(tmp_path / "py") + "/")
    r = subprocess.run([exe, "full", str(tmp_path / "in"), str(tmp_path / "cpp")], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    f32 = spec["dtype"] == "f"
    step_cpp, step_py = compare_folders(str(tmp_path / "cpp"), str(tmp_path / "py"), True,
                                        1e-6 if f32 else 1e-11, 1e-6 if f32 else 1e-9)
    assert abs(step_cpp - step_py) <= 1e-6 * step_py
    assert abs(float(r.stdout.split()[0]) - step_cpp) <= 1e-7 * step_cpp
    # the completed folder solves: FP64 SPOCK from a feasible state
    t = sg.ScenarioTree(str(tmp_path / "cpp"))
    c = sg.CacheBuilder(t, sg.ProblemData(t)).tol(1e-6).maxIters(2000).build()
    assert c.runSpock(np.zeros(spec["nx"])) in (0, 1)


@pytest.mark.gpu
def test_python_factory_gpu_offline_at_config2_size(exe, tmp_path):
    """Config-2 size (607 nodes, nx 50, nu 20): the Python factory with the GPU offline cache
    equals the numpy/ARPACK one, and the C++ generator writes the same folder.  Prints the
    three generation times."""
    from spock_gb300 import configs
    t0 = time.perf_counter()
    configs.config2(str(tmp_path / "host") + "/")
    t_host = time.perf_counter() - t0
    t0 = time.perf_counter()
    configs.config2(str(tmp_path / "gpu") + "/", offline="gpu")
    t_gpu = time.perf_counter() - t0
    s_gpu, s_host = compare_folders(str(tmp_path / "gpu"), str(tmp_path / "host"), True, 0., 1e-9)
    assert abs(s_gpu - s_host) <= 1e-6 * s_host
    spec, arr = make_case("cfg2")
    write_inputs(str(tmp_path / "in"), spec, arr)
    python_factory(spec, arr, str(tmp_path / "py") + "/")
    t0 = time.perf_counter()
    r = subprocess.run([exe, "full", str(tmp_path / "in"), str(tmp_path / "cpp")], capture_output=True, text=True,
                       timeout=600)
    t_cpp = time.perf_counter() - t0
    assert r.returncode == 0, r.stderr
    s_cpp, s_py = compare_folders(str(tmp_path / "cpp"), str(tmp_path / "py"), True, 1e-11, 1e-9)
    assert abs(s_cpp - s_py) <= 1e-6 * s_py
    print(f"\nconfig-2 generation: python+numpy/ARPACK {t_host:.2f} s, python+GPU cache {t_gpu:.2f} s, "
          f"C++ generator+GPU cache {t_cpp:.2f} s")


def _record_golden_inputs(case, monkeypatch, tmp_path):
    """Run test_factory's builder of a golden case with the tree classes and the problem writer
    intercepted: the raw inputs it passes (tree parameters, per-event dynamics and costs,
    constraints, risk, preconditioning) become a spec for the C++ driver."""
    import test_factory as TF
    rec = {}

    class Markov(F.MarkovChain):
        def __init__(self, P, v, horizon, stopping_stage=None):
            rec["tree"] = ("markov", np.asarray(P, float), np.asarray(v, float), horizon, stopping_stage)
            super().__init__(P, v, horizon, stopping_stage)

    class Iid(F.IidProcess):
        def __init__(self, d, horizon, stopping_stage=None):
            rec["tree"] = ("iid", np.asarray(d, float), horizon, stopping_stage)
            super().__init__(d, horizon, stopping_stage)

    def capture(self, path, dt="d", step_size=None, offline="host", device=0):
        rec["factory"] = self

    monkeypatch.setattr(F, "MarkovChain", Markov)
    monkeypatch.setattr(F, "IidProcess", Iid)
    monkeypatch.setattr(F.Factory, "generate_problem", capture)
    TF.BUILDERS[case](str(tmp_path / "unused") + "/")
    f, tr = rec["factory"], rec["tree"]
    ne = len(f.dyn_events)
    spec = dict(nx=f.nx, nu=f.nu, events=ne, dynamics="affine" if f.dyn_events[0].affine else "linear",
                cost=f.cost_events[0].kind, leaf=f.leaf_cost.kind, nlcon=f.nl_con.kind, lcon=f.l_con.kind,
                alpha=float(f.risk.alpha), precondition=int(bool(f.precondition)), scale=float(f.cost_scale), dtype="d")
    if tr[0] == "markov":
        spec.update(tree="markov", horizon=tr[3], stopping=tr[4] if tr[4] is not None else tr[3])
        arr = dict(tree_P=tr[1], tree_v=tr[2])
    else:
        spec.update(tree="iid", horizon=tr[2], stopping=tr[3] if tr[3] is not None else tr[2])
        arr = dict(tree_d=tr[1])
    z = lambda shape: np.zeros(shape)
    arr.update(dyn_A=np.array([d.A for d in f.dyn_events]), dyn_B=np.array([d.B for d in f.dyn_events]),
               dyn_c=np.array([d.c for d in f.dyn_events])[:, :, None])
    ce = f.cost_events
    arr.update(cost_Q=np.array([c.Q if c.Q is not None else z((f.nx, f.nx)) for c in ce]),
               cost_R=np.array([c.R if c.R is not None else z((f.nu, f.nu)) for c in ce]),
               cost_q=np.array([c.q if c.q is not None else z(f.nx) for c in ce])[:, :, None],
               cost_r=np.array([c.r if c.r is not None else z(f.nu) for c in ce])[:, :, None],
               leaf_Q=(f.leaf_cost.Q if f.leaf_cost.Q is not None else z((f.nx, f.nx)))[None],
               leaf_q=f.leaf_cost.q if f.leaf_cost.q is not None else z(f.nx))
    for p, con in (("nl_", f.nl_con), ("l_", f.l_con)):
        if con.kind in ("rectangle", "polyhedronWithIdentity", "rectangleInputBall"):
            n_id = con.nx if con.kind == "rectangleInputBall" else con.lb.size
            arr.update({p + "lb": con.lb[:n_id], p + "ub": con.ub[:n_id]})
        if con.kind in ("polyhedron", "polyhedronWithIdentity"):
            arr.update({p + "G": con.G, p + "glb": con.glb if con.kind == "polyhedronWithIdentity" else con.lb,
                        p + "gub": con.gub if con.kind == "polyhedronWithIdentity" else con.ub})
        if con.kind == "rectangleInputBall":
            spec["radius"] = con.radius
    return spec, arr


@pytest.mark.parametrize("case", ["reftest", "cfg1", "qpl", "affpoly"])
def test_cpp_problem_data_matches_reference_golden(exe, tmp_path, monkeypatch, case):
    """The C++ generator on the raw inputs of a golden case against the folder the reference's
    own Python factory wrote (tests/golden/<case>): every problem-data tensor (the offline cache
    aside) and every data.json key but the step size."""
    from conftest import GOLDEN
    spec, arr = _record_golden_inputs(case, monkeypatch, tmp_path)
    write_inputs(str(tmp_path / "in"), spec, arr)
    r = subprocess.run([exe, "data", str(tmp_path / "in"), str(tmp_path / "cpp")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    ref_dir, mine = os.path.join(GOLDEN, case), str(tmp_path / "cpp")
    ref_files = sorted(f for f in os.listdir(ref_dir) if f.endswith(".bt") and not f.startswith(("test_", "initialState"))
                       and f.rsplit("_", 1)[0] not in CACHE)
    assert sorted(f for f in os.listdir(mine) if f.endswith(".bt")) == ref_files
    for f in ref_files:
        (a, da), (b, db) = read_bt(os.path.join(ref_dir, f)), read_bt(os.path.join(mine, f))
        assert da == db, f
        if f.endswith("_u.bt"):
            assert np.array_equal(a, b), f
            continue
        # the reference's sqrtm of the root's all-zero cost matrix (never read) is not finite
        fin = np.isfinite(a)
        scale = max(1., np.abs(a[fin]).max()) if fin.any() else 1.
        assert np.abs(a[fin] - b[fin]).max(initial=0.) <= 1e-10 * scale, f
    ref_meta = json.load(open(os.path.join(ref_dir, "data.json")))
    meta = json.load(open(os.path.join(mine, "data.json")))
    for k, v in ref_meta.items():
        if k not in ("stepSize", "rowsS2"):
            assert meta[k] == v, k


def test_gpu_offline_cache_fails_loudly_without_a_gpu(tmp_path):
    """The offline cache is GPU code with no host fallback: without a device the Python factory's
    offline="gpu" path raises, after writing the problem data."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    sg.build()
    spec, arr = make_case("cfg1")
    with pytest.raises(RuntimeError):
        python_factory(spec, arr, str(tmp_path / "p") + "/", offline="gpu")
    assert os.path.exists(tmp_path / "p" / "dynamics_AB_d.bt")
    assert not os.path.exists(tmp_path / "p" / "dynamics_P_d.bt")
