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
    assert L.pps_abi_version() == 1
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
])
def test_invalid_arguments_are_rejected_before_any_device_work(pps_lib, bad):
    L = pps_lib.load()
    g = pps_lib.BlockGrid(npglobal=bad.get("npglobal", (10, 10, 10)), ds=bad.get("ds", (0.1, 0.1, 0.1)),
                          bcs=bad.get("bcs", (0,) * 6)).c()
    cfg = pps_lib.PpsConfig()
    L.pps_config_default(C.byref(cfg), 0)
    for k in ("krylov", "precond", "cheb_degree", "maxit", "tol", "form", "inner_tol"):
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
