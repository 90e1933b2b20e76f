"""One capped solve of the benchmark workload, sized for profiling.

    python -m parallelpoissonsolver_gb300.profile_case --size 320 --form mixed --maxit 2

Runs `--repeat` solves of the k^-2 random-field workload at `--size`^3 unknowns with
the iteration cap `--maxit`, so that an ncu capture sees a handful of launches of
every kernel of the loop on fields larger than L2, and exits 0 whether or not the
cap stops the solve.
"""
from __future__ import annotations

import argparse

import parallelpoissonsolver_gb300 as pps
from parallelpoissonsolver_gb300 import workloads


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=320)
    ap.add_argument("--form", default="mixed", choices=list(pps.FORMS))
    ap.add_argument("--maxit", type=int, default=2)
    ap.add_argument("--degree", type=int, default=11)
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--graph", action="store_true")
    a = ap.parse_args()
    grid = pps.BlockGrid.cube(a.size)
    b = workloads.random_field(a.size, seed=2)
    s = pps.BiCGSTAB(grid, pps.ChebyshevIteration(a.degree), tolerance=1e-10, max_iteration=a.maxit,
                     form=a.form, inner_maxit=a.maxit, max_refinements=1, use_graph=a.graph)
    for _ in range(a.repeat):
        x = grid.new_field()
        st = s(x, b.copy(), raise_on_error=True)
        d = s.stats()
        print(f"status {pps.status_string(st)}: {d['iterations']} iterations, {d['kernel_launches']} launches, "
              f"{d['seconds_solve'] * 1e3:.2f} ms, sweep {d['sweep_bytes'] / max(d['sweep_seconds'], 1e-12) / 1e9:.0f} GB/s")
    s.close()


if __name__ == "__main__":
    main()
