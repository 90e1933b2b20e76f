"""The drop-in boundary, built: the reference's own driver, solverPoissonMPI_CPU/src/
main.cpp, compiles UNCHANGED against the libpps C++ shim with only the composition
alias swapped (oracle/dropin/inputParam.hpp; `make -C oracle dropin`) and links to
libpps.so.  Without a GPU the run reaches the solver's constructor (pps_create) and
stops there with the library's no-device error; tests/test_gpu_dropin.py runs it to
the end on a GPU.  Skipped where the reference sources are not mounted."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_dropin(pps_lib, O):
    if not (O.REF_INCLUDE and os.path.isfile(os.path.join(O.REF_INCLUDE, "..", "src", "main.cpp"))):
        pytest.skip("the reference sources (solverPoissonMPI_CPU) are not mounted here")
    pps_lib.lib_path()
    r = subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "dropin", f"REF_INCLUDE={O.REF_INCLUDE}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return os.path.join(ROOT, "oracle", "_ref", "dropin_main")


def test_reference_driver_builds_and_reaches_the_gpu(pps_lib, oracle):
    exe = build_dropin(pps_lib, oracle)
    r = subprocess.run([exe, "1", "1", "1"], capture_output=True, text=True, timeout=600)
    assert "Global grid size from block 66 66 66" in r.stdout
    if pps_lib.device_count() == 0:
        assert r.returncode != 0 and "pps_create: no CUDA device" in r.stderr, (r.stdout, r.stderr)
    else:
        assert r.returncode == 0, r.stderr
        assert "Iterative solver finished with iter:" in r.stdout
