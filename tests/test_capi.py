"""The C-ABI library builds, loads and exports every entry point of include/*.h; host-only
calls (data-folder loading and its error behaviour) work without a GPU."""
import ctypes
import glob
import os
import re
import shutil

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

import spock_gb300 as sg


@pytest.fixture(scope="module")
def built():
    sg.build()
    return sg.lib()


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        names |= set(re.findall(r"\b(spock_\w+)\s*\(", text))
    return sorted(names)


def test_exports_every_declared_symbol(built):
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(built, n), n


def test_load_sizes_match_oracle(built, oracle_lib):
    for case in ["reftest", "cfg1", "qpl", "affpoly"]:
        t = sg.ScenarioTree(os.path.join(GOLDEN, case))
        d = sg.ProblemData(t)
        P = oracle_lib.Problem(os.path.join(GOLDEN, case))
        assert (t.numNodes(), t.numNonleafNodes(), t.numStages(), t.numStates(), t.numInputs(), t.numEvents()) == \
            (P.n, P.nnl, P.ns, P.nx, P.nu, P.ne)
        assert (t._sp, t._sd) == (P.size_prim, P.size_dual)
        assert d.stepSize() == P.step
        assert np.array_equal(d.scaling(), P.scaling)


def test_load_errors(built, tmp_path):
    with pytest.raises(ValueError, match="cannot open"):
        sg.ScenarioTree(str(tmp_path / "missing"))
    bad = tmp_path / "bad"
    shutil.copytree(os.path.join(GOLDEN, "cfg1"), bad)
    with open(bad / "data.json", "w") as fh:
        fh.write('{"numEvents": 3, "numNodes": 31}')
    with pytest.raises(ValueError, match="missing key"):
        sg.ScenarioTree(str(bad))
    short = tmp_path / "short"
    shutil.copytree(os.path.join(GOLDEN, "cfg1"), short)
    with open(short / "dynamics_K_d.bt", "r+b") as fh:
        fh.truncate(40)
    with pytest.raises(ValueError, match="dynamics_K"):
        sg.ScenarioTree(str(short))
    risk = tmp_path / "risk"
    shutil.copytree(os.path.join(GOLDEN, "cfg1"), risk)
    txt = open(risk / "data.json").read().replace('"avar"', '"evar"')
    open(risk / "data.json", "w").write(txt)
    with pytest.raises(ValueError, match="Risk type evar is not supported"):
        sg.ScenarioTree(str(risk))


def test_options_defaults(built):
    o = sg.Options()
    built.spock_options_default(ctypes.byref(o))
    assert (o.tol_abs, o.tol_rel, o.max_iters, o.max_inner, o.anderson, o.precision, o.batch) == \
        (1e-3, 0., 0, 8, 3, 64, 1)
