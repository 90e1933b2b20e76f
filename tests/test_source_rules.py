"""Rules the CUDA sources rely on for stream ordering, checked on the text (CPU).

- Every kernel is launched with programmatic dependent launch, so every kernel must
  begin with pdl_enter(): it waits for the kernel before it on the stream before any
  global memory access.  A kernel without it could read its predecessor's output early.
- The library's streams are non-blocking, so the legacy default stream is not ordered
  with their kernels: no synchronous cudaMemcpy anywhere, and cudaMemset only in the
  solver's constructor, which synchronises the device before it returns.
"""
import os
import re

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "parallelpoissonsolver_gb300",
                    "csrc")
SOURCES = sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh")))


def read(name):
    with open(os.path.join(CSRC, name)) as f:
        return f.read()


def test_every_kernel_waits_for_its_predecessor_first():
    missing = []
    count = 0
    for name in SOURCES:
        text = read(name)
        for m in re.finditer(r"__global__", text):
            body = text.index("{", m.end())
            first = text[body + 1:].lstrip()
            count += 1
            if not first.startswith("pdl_enter();"):
                line = text.count("\n", 0, m.start()) + 1
                missing.append(f"{name}:{line}")
    assert count > 50
    assert not missing, missing


def test_launches_go_through_launch_pdl():
    chevrons = [f"{name}:{text.count(chr(10), 0, m.start()) + 1}"
                for name in SOURCES for text in [read(name)] for m in re.finditer(r"<<<", text)]
    assert not chevrons, chevrons


def test_no_legacy_stream_copies_or_fills_outside_the_constructor():
    sync_copies = [name for name in SOURCES if re.search(r"\bcudaMemcpy\(", read(name))]
    assert not sync_copies, sync_copies
    fills = [name for name in SOURCES if re.search(r"\bcudaMemset\(", read(name))]
    assert fills == ["pps_solver.cu"], fills
    text = read("pps_solver.cu")
    create = text.index("pps_status pps_create(")
    end = text.index("CK(cudaDeviceSynchronize());", create)
    outside = [m.start() for m in re.finditer(r"\bcudaMemset\(", text) if not (create < m.start() < end)]
    # alloc_fields, called from pps_create only, holds the other fills
    helper = text.index("void alloc_fields(")
    helper_end = text.index("\n}\n", helper)
    assert all(helper < p < helper_end for p in outside), outside
    assert text.count("alloc_fields<") == text[create:end].count("alloc_fields<")
