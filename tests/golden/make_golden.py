"""Generate the golden fixtures in tests/golden/ from the REFERENCE's own solver.

Runs each case of cases.py through oracle/_ref/libppsref.so -- the reference's
solverPoissonMPI_CPU headers compiled unchanged by `make -C oracle ref` -- and
stores inputs and outputs (or, for the 64^3 cases, a summary with checksums and a
sample).  It also checks, before writing, that the C restatement in
oracle/pps_oracle.c reproduces every output bit for bit.

Usage (needs the reference sources, so it runs where they are mounted):
    python tests/golden/make_golden.py [case name ...]     (default: every case)
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle import oracle as O  # noqa: E402
from cases import CASES, random_inputs  # noqa: E402

SAMPLE = 4096


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def make_inputs(case):
    grid = O.Grid(np=case["np"], ds=case["ds"], origin=case["origin"], bcs=case["bcs"])
    kind, arg = case["inputs"]
    if kind == "problem":
        x, b, faces = O.set_problem(grid, arg)
        if not any(f is not None for f in faces):
            faces = None
        return grid, x, b, faces, arg
    x, b, faces = random_inputs(case, arg)
    if not any(f is not None for f in faces):
        faces = None
    if kind == "warm":
        # converge once to a tight tolerance, then use that solution as the initial guess
        c = O.Config(**{**case["cfg"], "tol": 1e-13, "maxit": 20000})
        xs, bs = x.copy(), b.copy()
        O.solve(grid, c, xs, bs, faces)
        x = xs
    return grid, x, b, faces, None


def run_case(case):
    grid, x0, b0, faces, problem = make_inputs(case)
    cfg = O.Config(**case["cfg"])
    xr, br = x0.copy(), b0.copy()
    ref = O.ref_solve(grid, cfg, xr, br, problem=problem if problem is not None else 0, neumann=faces)
    xp, bp = x0.copy(), b0.copy()
    port = O.solve(grid, cfg, xp, bp, faces)
    bits = lambda a: np.asarray(a, np.float64).view(np.uint64)  # noqa: E731  (NaN-aware, bit for bit)
    same = (np.array_equal(bits(xr), bits(xp)) and np.array_equal(bits(br), bits(bp))
            and ref.iterations == port.iterations and np.array_equal(bits(ref.history), bits(port.history))
            and bits(ref.err_true) == bits(port.err_true))
    if not same:
        raise SystemExit(f"{case['name']}: the C restatement differs from the reference")
    theta, delta, sigma = O.cheb_params(grid, cfg)
    out = dict(iterations=ref.iterations, err_iter=ref.err_iter, err_true=ref.err_true, history=ref.history,
               theta=theta, delta=delta, sigma=sigma, x_in_sha=sha(x0), b_in_sha=sha(b0), x_out_sha=sha(xr),
               b_out_sha=sha(br))
    if case["store"] == "full":
        out.update(x_in=x0, b_in=b0, x_out=xr, b_out=br)
        if faces is not None:
            for f, a in enumerate(faces):
                if a is not None:
                    out[f"face{f}"] = a
    else:
        rng = np.random.default_rng(0)
        idx = rng.integers(0, xr.size, SAMPLE)
        out.update(sample_index=idx, x_out_sample=xr.ravel()[idx], x_out_sum=float(xr.sum()),
                   x_out_l2=float(np.sqrt((xr * xr).sum())))
    return out


def main():
    O.build(ref=True)
    names = set(sys.argv[1:])
    for case in CASES:
        if names and case["name"] not in names:
            continue
        out = run_case(case)
        path = os.path.join(HERE, case["name"] + ".npz")
        np.savez_compressed(path, **out)
        print(f"{case['name']:32s} iterations {out['iterations']:5d} err_true {out['err_true']:.3e}  "
              f"{os.path.getsize(path) / 1024:.0f} KiB")


if __name__ == "__main__":
    main()
