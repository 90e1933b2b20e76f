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

The spread: BiCGSTAB's iteration count on this workload is chaotic in rounding.
The same solve on copies of b changed by one ulp in 1% of its entries (seeds
--spread-first .. --spread-first + --spread - 1) gives the reference's own range of
counts and how far apart its solutions land; those runs use the oracle's C
restatement (bit-identical to the reference, faster with threads).  A solver that
rounds differently, or a b built by another FFT library, is one more such
perturbation.

Usage (needs the reference sources; one core, about 13 s per reference iteration
at 512^3):
    python tests/golden/make_record_512.py [--m 512] [--tols 1e-10,1e-13] [--spread 4]
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
    ap.add_argument("--spread", type=int, default=4, help="perturbed solves at tolerance 1e-10")
    ap.add_argument("--spread-first", type=int, default=1, help="seed of the first perturbation")
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--out", default=os.path.join(HERE, "record_512.npz"))
    args = ap.parse_args()
    O.build(ref=True)
    m = args.m
    grid = O.cube(m)
    b0 = workloads.random_field(m, seed=2, device="cpu")
    idx = sample_index(m)
    out = dict(m=m, sample_index=idx, b_sha=hashlib.sha256(b0.tobytes()).hexdigest(),
               b_l2=float(np.sqrt((b0 * b0).sum())), b_sample=b0.ravel()[idx])
    for tol in [float(t) for t in args.tols.split(",") if t]:
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
    its, seeds, samples = [], [], []
    for seed in range(args.spread_first, args.spread_first + args.spread):
        b = b0.copy()
        mask = np.random.default_rng(seed).random(b.shape) < 0.01
        b[mask] = np.nextafter(b[mask], np.inf)
        x = np.zeros_like(b0)
        r = O.solve(grid, O.Config(**{**O.CPU_PRESET, "tol": 1e-10, "maxit": 1700, "threads": args.threads}), x, b)
        its.append(r.iterations)
        seeds.append(seed)
        samples.append(x.ravel()[idx])
        print(f"perturbation {seed}: {r.iterations} iterations", flush=True)
        del x, b
    if its:
        out.update(spread_seeds=np.array(seeds), spread_iterations=np.array(its), spread_x_sample=np.array(samples))
    np.savez_compressed(args.out, **out)
    print(f"wrote {args.out} ({os.path.getsize(args.out) / 1024:.0f} KiB)")


if __name__ == "__main__":
    main()
