"""The drop-in boundary on the GPU, through the C++ shim (include/pps_solver.hpp).

* tests/shim_driver.cpp makes the reference driver's calls (main.cpp:83-127:
  constructor, setProblem, operator()(x, b, A), the getters,
  checkSolutionLocalGlobal) with stand-ins for the reference's grid, problem,
  communicator and operator types; built here with g++ against libpps.so and run:
  in the PARITY form its iteration count, both errors and x are bit-identical to the
  oracle's (the reference's own classes, compiled where they lie, agree with the
  oracle bit for bit), in the FP64 form within the reassociation envelope.
* Where the reference sources are mounted, the reference's main.cpp itself, built
  unchanged against the shim (`make -C oracle dropin`), runs the same problem and
  prints the oracle's iteration count.
"""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

import parallelpoissonsolver_gb300 as pps
from conftest import rel_l2, same_bits
from test_dropin_cpu import build_dropin

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LINE = re.compile(r"Iterative solver finished with iter: (\d+) error from algo (\S+) error r=b-Ax (\S+)")


def oracle_run(O, m):
    g = O.cube(m)
    x, b, _ = O.set_problem(g, 0)
    r = O.solve(g, O.Config(tol=100 * 1e-10, maxit=1700, threads=4), x, b)   # tollMainSolver = 1e2
    return r, x


@pytest.fixture(scope="module")
def driver(gpu, tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    exe = str(tmp_path_factory.mktemp("shim") / "shim_driver")
    lib = os.path.dirname(pps.lib_path())
    r = subprocess.run([gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), "-o", exe,
                        os.path.join(ROOT, "tests", "shim_driver.cpp"), "-L", lib, "-lpps", f"-Wl,-rpath,{lib}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("form", ["parity", "fp64"])
def test_shim_driver_matches_the_oracle(driver, oracle, tmp_path, form):
    m = 40
    sol = str(tmp_path / "solution.dat")
    r = subprocess.run([driver, str(m), form, sol], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    it, e_iter, e_true = LINE.search(r.stdout).groups()
    ref, x_ref = oracle_run(oracle, m)
    x = np.fromfile(sol, dtype="<f8").reshape(x_ref.shape)
    if form == "parity":
        assert int(it) == ref.iterations
        assert float(e_iter) == ref.err_iter and float(e_true) == ref.err_true
        assert same_bits(x, x_ref)
    else:
        assert abs(int(it) - ref.iterations) <= 1
        assert float(e_true) <= 1e-8
        assert rel_l2(x, x_ref) <= 1e-9
    assert "Max error local point" in r.stdout


def test_reference_main_on_the_shim(gpu, pps_lib, oracle):
    exe = build_dropin(pps_lib, oracle)
    ref, _ = oracle_run(oracle, 64)
    for form in ("parity", "fp64"):
        r = subprocess.run([exe, "1", "1", "1"], capture_output=True, text=True, timeout=600,
                           env=dict(os.environ, PPS_FORM=form))
        assert r.returncode == 0, r.stderr
        it = int(LINE.search(r.stdout).group(1))
        assert it == ref.iterations if form == "parity" else abs(it - ref.iterations) <= 1
