"""The C++ interface (include/spock_gb300.hpp), compiled with g++ against the C-ABI library the
way a user program is (tests/cpp/wrapper_main.cpp): host-side loading and its errors on the CPU,
an FP64 solve against the oracle on the GPU."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

import spock_gb300 as sg


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    lib = sg.build()
    out = str(tmp_path_factory.mktemp("cpp") / "wrapper_main")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "wrapper_main.cpp"), "-o", out,
                           "-L", os.path.dirname(lib), "-lspock_gb300",
                           "-Wl,-rpath," + os.path.dirname(lib)])
    return out


def run(exe, *args):
    return subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, timeout=600)


@pytest.mark.parametrize("case", ["reftest", "cfg1", "qpl"])
def test_tree_and_problem_load(exe, oracle_lib, case):
    path = os.path.join(GOLDEN, case)
    r = run(exe, "load", path)
    assert r.returncode == 0, r.stderr
    ne, n, nnl, ns, nx, nu, step = r.stdout.split()
    P = oracle_lib.Problem(path)
    assert (int(n), int(nnl), int(nx), int(nu)) == (P.n, P.nnl, P.nx, P.nu)
    assert float(step) == P.step


def test_missing_folder_throws_invalid_argument(exe, tmp_path):
    r = run(exe, "bad", str(tmp_path / "nowhere"))
    assert r.returncode == 0 and r.stdout.startswith("invalid_argument"), r.stdout + r.stderr


@pytest.mark.gpu
def test_cpp_solve_matches_oracle(exe, oracle_lib):
    """Cache<double>::runSpock to 1e-10 on the reference's test problem (testCache.cu:294-308)
    through the C++ interface: converged, and u_0 agrees with the oracle to 1e-8."""
    path = os.path.join(GOLDEN, "reftest")
    P = oracle_lib.Problem(path)
    x0 = np.full(P.nx, 1.1)
    r = run(exe, "solve", path, 1e-10, *x0)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.split("\n")
    status, iters = int(lines[0].split()[0]), int(lines[0].split()[1])
    assert status == 0 and iters > 0
    u0 = np.array([float(v) for v in lines[1:1 + P.nu]])
    assert lines[1 + P.nu].startswith("getDual") and float(lines[1 + P.nu].split()[1]) < 1e-6
    z, s = P.run(x0, oracle_lib.options(tol=1e-10, max_iters=20000), "spock")
    u_ref = P.states_inputs(z)[1][:P.nu]
    assert np.abs(u0 - u_ref).max() <= 1e-8 * max(1., np.abs(u_ref).max())
