"""In-tree build of libpps.so (nvcc, sm_103a only).

The seven translation units of csrc/ (kernels, solver, allocation-free entry point,
batched solves per phase and in one persistent launch, U-Net kernels and U-Net host
code) compile in parallel, one
-gencode for sm_103a, and link into ``parallelpoissonsolver_gb300/libpps.so``
beside this file.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpps.so")
SOURCES = ["pps_kernels.cu", "pps_solver.cu", "pps_noalloc.cu", "pps_batch.cu", "pps_bvcycle.cu",
           "pps_unet_kernels.cu", "pps_unet.cu"]
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              # host code rounds every product and sum separately (aarch64 g++ would fuse them)
              "-Xcompiler", "-ffp-contract=off"] + GENCODE


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: libpps needs the CUDA toolkit to build")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile libpps.so if any source or header is newer than it. Returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "pps.h"))
    headers.append(os.path.abspath(__file__))   # flags live here
    nv = nvcc()
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nv, *NVCC_FLAGS, "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        run([nv, "-shared", *GENCODE, "-o", LIB, *objs])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
