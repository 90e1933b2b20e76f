"""Reference record of the 512^3 random-field solve, made by the REFERENCE's own solver.

The workload: 512^3 interior unknowns, h = 1/513, Dirichlet 0, b = -f for f the
seeded k^-2 Gaussian random field of parallelpoissonsolver_gb300.workloads
(seed 2, unit RMS, generated on the CPU), solved by the reference's BiCGSTAB with
its Chebyshev(11) preconditioner (CPU preset, solverSetup.hpp) through
oracle/_ref/libppsref.so -- the solverPoissonMPI_CPU headers compiled unchanged by
`make -C oracle ref` (BiCGSTAB.hpp:55-322).  Two stop tolerances: 1e-10 (the
benchmark's) and 1e-13 (the tolerance at which two correct FP64 solvers agree to
about 1e-13 in relative L2).

Stored per tolerance (record_512.npz): the iteration count, the residual history,
the recursive and true normalised residuals, the L2 norm and sum of x over the
whole field, and x at a fixed sample of 32,768 unknowns; once: b's checksum, its
L2 norm and b at the same sample, so a run elsewhere can tell how close its own
copy of the input is (FFT libraries differ in the last bits between machines).

Usage (needs the reference sources; one core, about 16 s per iteration at 512^3):
    python tests/golden/make_record_512.py [--m 512] [--tols 1e-10,1e-13]
"""
from __future__ import annotations

import argparse
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from parallelpoissonsolver_gb300 import workloads  # noqa: E402

SAMPLE = 32768


def sample_index(m: int) -> np.ndarray:
    """Flat indices of SAMPLE unknowns of the guard-padded (m+4)^3 field, in order."""
    rng = np.random.default_rng(512)
    n = m + 4
    k = rng.integers(2, m + 2, SAMPLE)
    j = rng.integers(2, m + 2, SAMPLE)
    i = rng.integers(2, m + 2, SAMPLE)
    return np.sort(i + n * (j + n * k)).astype(np.int64)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--m", type=int, default=512)
    ap.add_argument("--tols", default="1e-10,1e-13")
    ap.add_argument("--out", default=os.path.join(HERE, "record_512.npz"))
    args = ap.parse_args()
    O.build(ref=True)
    m = args.m
    grid = O.cube(m)
    b0 = workloads.random_field(m, seed=2, device="cpu")
    idx = sample_index(m)
    out = dict(m=m, sample_index=idx, b_sha=hashlib.sha256(b0.tobytes()).hexdigest(),
               b_l2=float(np.sqrt((b0 * b0).sum())), b_sample=b0.ravel()[idx])
    for tol in [float(t) for t in args.tols.split(",")]:
        tag = f"{tol:.0e}".replace("-", "m")
        x = np.zeros_like(b0)
        b = b0.copy()
        cfg = O.Config(**{**O.CPU_PRESET, "tol": tol, "maxit": 1700})
        t0 = time.perf_counter()
        r = O.ref_solve(grid, cfg, x, b)
        wall = time.perf_counter() - t0
        out.update({f"{tag}_iterations": r.iterations, f"{tag}_history": r.history, f"{tag}_err_iter": r.err_iter,
                    f"{tag}_err_true": r.err_true, f"{tag}_x_l2": float(np.sqrt((x * x).sum())),
                    f"{tag}_x_sum": float(x.sum()), f"{tag}_x_sample": x.ravel()[idx],
                    f"{tag}_seconds": wall})
        print(f"tol {tol:.0e}: {r.iterations} iterations, err_iter {r.err_iter:.3e}, err_true {r.err_true:.3e}, "
              f"{wall:.0f} s", flush=True)
        del x, b
    np.savez_compressed(args.out, **out)
    print(f"wrote {args.out} ({os.path.getsize(args.out) / 1024:.0f} KiB)")


if __name__ == "__main__":
    main()
