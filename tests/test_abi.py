"""The C ABI boundary on the CPU: the library loads, exports every symbol that
include/*.h declares, validates its arguments without touching a GPU, and the C++
class shim compiles."""
import ctypes as C
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def declared_symbols():
    names = set()
    for fn in os.listdir(INCLUDE):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(INCLUDE, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(pps_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_the_entry_points():
    names = declared_symbols()
    for n in ("pps_create", "pps_solve", "pps_solve_device", "pps_destroy", "pps_set_problem"):
        assert n in names


def test_library_exports_every_declared_symbol(pps_lib):
    L = C.CDLL(pps_lib.lib_path())
    missing = [n for n in declared_symbols() if not hasattr(L, n)]
    assert not missing, missing
    assert sorted(set(pps_lib.EXPORTED) - set(declared_symbols())) == []


def test_abi_version_and_status_strings(pps_lib):
    L = pps_lib.load()
    assert L.pps_abi_version() == 3
    for st in (0, 1, 2, 3, 4, -1, -2, -3, -4, -5, -6):
        assert pps_lib.status_string(st) not in ("", "unknown status")


def test_presets_match_reference_constants(pps_lib):
    cfg = pps_lib.PpsConfig()
    L = pps_lib.load()
    assert L.pps_config_default(C.byref(cfg), pps_lib.PRESET_CPU) == 0
    # solverSetup.hpp:22,27-28,37-40 of the CPU code
    assert (cfg.cheb_degree, cfg.cheb_eps, cfg.rescale_min, cfg.maxit) == (11, 1e-4, 500.0, 1700)
    assert cfg.rescale_max == 1 - 1e-4 and cfg.tol == 100 * 1e-10
    assert L.pps_config_default(C.byref(cfg), pps_lib.PRESET_ALPAKA) == 0
    # ALP/include/solverSetup.hpp:52,58-59,68-71
    assert (cfg.cheb_degree, cfg.cheb_eps, cfg.rescale_min, cfg.maxit, cfg.tol) == (24, 0.0, 100.0, 1000, 1e-10)
    # the inner-solver preconditioner: tollPreconditionerSolver = tollMainSolver * 1e8, 500 iterations
    assert (cfg.precond_tol, cfg.precond_maxit, cfg.precond_inner) == (1e8 * 1e-10, 500, pps_lib.PREC_NONE)
    assert L.pps_config_default(C.byref(cfg), pps_lib.PRESET_CPU) == 0
    # CPU solverSetup.hpp:31-33: tollPreconditionerSolver 1e4, iterMaxPreconditioner 150
    assert (cfg.precond_tol, cfg.precond_maxit) == (1e4 * 1e-10, 150)
    assert L.pps_config_default(C.byref(cfg), 7) == pps_lib.ERR_INVALID_ARG


@pytest.mark.parametrize("bad", [
    dict(npglobal=(2, 10, 10)),
    dict(ds=(0.0, 0.1, 0.1)),
    dict(bcs=(0, 2, 0, 0, 0, 0)),
    dict(krylov=5),
    dict(precond=9),
    dict(cheb_degree=0),
    dict(maxit=-1),
    dict(tol=-1.0),
    dict(form=7),
    dict(form=2, inner_tol=1.5),
    dict(precond=4),
    dict(precond=2, precond_tol=1.5),
    dict(precond=3, precond_tol=0.0),
    dict(precond=2, precond_inner=2),
    dict(precond=3, precond_maxit=-1),
    dict(precond=2, precond_inner=1, cheb_degree=0),
    dict(krylov=3, cheb_degree=0),
    dict(krylov=3, cheb_degree=10001),
])
def test_invalid_arguments_are_rejected_before_any_device_work(pps_lib, bad):
    L = pps_lib.load()
    g = pps_lib.BlockGrid(npglobal=bad.get("npglobal", (10, 10, 10)), ds=bad.get("ds", (0.1, 0.1, 0.1)),
                          bcs=bad.get("bcs", (0,) * 6)).c()
    cfg = pps_lib.PpsConfig()
    L.pps_config_default(C.byref(cfg), 0)
    for k in ("krylov", "precond", "cheb_degree", "maxit", "tol", "form", "inner_tol", "precond_tol",
              "precond_maxit", "precond_inner"):
        if k in bad:
            setattr(cfg, k, bad[k])
    h = C.c_void_p()
    assert L.pps_create(C.byref(g), C.byref(cfg), C.byref(h)) == pps_lib.ERR_INVALID_ARG
    assert not h.value
    assert pps_lib.last_error() != ""


def test_null_handles_are_rejected(pps_lib):
    L = pps_lib.load()
    assert L.pps_destroy(None) == pps_lib.ERR_INVALID_ARG
    assert L.pps_solve(None, None, None, None) == pps_lib.ERR_INVALID_ARG
    assert L.pps_get_history(None, None, 0, None) == pps_lib.ERR_INVALID_ARG


def test_create_without_gpu_fails_loudly(pps_lib):
    if pps_lib.device_count() > 0:
        pytest.skip("a GPU is visible")
    with pytest.raises(pps_lib.PpsError) as e:
        pps_lib.BiCGSTAB(pps_lib.BlockGrid.cube(8))
    assert e.value.status == pps_lib.ERR_NO_DEVICE


def test_cpp_shim_compiles():
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    src = os.path.join(ROOT, "include", "pps_solver.hpp")
    r = subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-x", "c++", "-I", INCLUDE, src],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


SHIM_COMPOSITIONS = r"""
#include <array>
#include "pps_solver.hpp"
struct Grid {
    std::array<int, 3> getNranks() const { return {1, 1, 1}; }
    std::array<int, 3> getNpglobal() const { return {10, 10, 10}; }
    std::array<double, 3> getDs() const { return {0.1, 0.1, 0.1}; }
    std::array<double, 3> getOrigin() const { return {0, 0, 0}; }
    std::array<int, 6> getBcsType() const { return {0, 0, 0, 0, 0, 0}; }
};
struct Exact {
    double setFieldB(double, double, double) const { return 0; }
    double trueSolutionFxyz(double, double, double) const { return 0; }
    double trueSolutionDdir(double, double, double, int) const { return 0; }
};
struct Comm {};
using None = pps::NoneSolver<3, double, 10000, 150>;
using Cheb = pps::ChebyshevIteration<3, double, 10000, 11, false, false, None>;
using InnerBiCG = pps::BiCGSTAB<3, double, 10000, 150, false, false, None>;
using InnerCG = pps::BaseCG<3, double, 10000, 150, false, false, Cheb>;
using S1 = pps::BiCGSTAB<3, double, 100, 1700, true, true, Cheb>;
using S2 = pps::BiCGSTAB<3, double, 100, 1700, true, true, InnerBiCG>;
using S3 = pps::BiCGSTAB<3, double, 100, 1700, true, true, InnerCG>;
using S4 = pps::ChebyshevIteration<3, double, 10000, 80, true, true, None>;
using S5 = pps::BaseCG<3, double, 100, 1700, true, true, InnerBiCG>;
static_assert(InnerBiCG::precond == PPS_PREC_BICGSTAB && InnerCG::precond == PPS_PREC_CG, "");
static_assert(InnerCG::inner_precond == PPS_PREC_CHEBYSHEV && InnerCG::degree == 11, "");
template <class S>
void use(const Grid& g, const Exact& e, Comm& c, double* x, double* b)
{
    S s(g, e, c);
    s.setProblem(x, b);
    s(x, b);
    (void)s.getNumIterationFinal();
    (void)s.getErrorComputeOperator();
    (void)s.getNumIterationPreconditionerFinal();
}
template void use<S1>(const Grid&, const Exact&, Comm&, double*, double*);
template void use<S2>(const Grid&, const Exact&, Comm&, double*, double*);
template void use<S3>(const Grid&, const Exact&, Comm&, double*, double*);
template void use<S4>(const Grid&, const Exact&, Comm&, double*, double*);
template void use<S5>(const Grid&, const Exact&, Comm&, double*, double*);
"""


def test_cpp_shim_instantiates_every_composition(tmp_path):
    """The type aliases of inputParam.hpp's compositions (main Chebyshev iteration,
    BiCGSTAB and CG as preconditioners) instantiate against the shim."""
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    src = tmp_path / "compositions.cpp"
    src.write_text(SHIM_COMPOSITIONS)
    r = subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-I", INCLUDE, str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_write_solution_host_field(pps_lib, tmp_path):
    """solution.dat (ALP/src/main.cpp:135-146): each rank's guard-padded field, raw
    doubles, at offset rank * G * 8; the file is not truncated, so ranks share it.
    Host fields need no GPU."""
    grid = pps_lib.BlockGrid(npglobal=(5, 4, 3), ds=(0.1, 0.1, 0.1))
    rng = __import__("numpy").random.default_rng(0)
    x0, x1 = rng.standard_normal(grid.shape), rng.standard_normal(grid.shape)
    path = str(tmp_path / "solution.dat")
    pps_lib.write_solution(grid, x1, path, rank=1)
    pps_lib.write_solution(grid, x0, path, rank=0)      # rank 0 after rank 1: no truncation
    data = __import__("numpy").fromfile(path, dtype="<f8")
    G = x0.size
    assert data.size == 2 * G
    assert (data[:G] == x0.ravel()).all() and (data[G:] == x1.ravel()).all()
    with pytest.raises(ValueError):
        pps_lib.write_solution(grid, x0[:-1], path)
