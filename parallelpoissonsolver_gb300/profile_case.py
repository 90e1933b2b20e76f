"""One capped solve of the benchmark workload, sized for profiling.

    python -m parallelpoissonsolver_gb300.profile_case --size 320 --form mixed --maxit 2
    python -m parallelpoissonsolver_gb300.profile_case --size 320 --krylov fcg --maxit 3
    python -m parallelpoissonsolver_gb300.profile_case --save-net net.npz          # train the U-Net, save
    python -m parallelpoissonsolver_gb300.profile_case --size 512 --learned net.npz --maxit 8
    python -m parallelpoissonsolver_gb300.profile_case --size 512 --learned net.npz --cycle 5,4,8 --maxit 20000 \
        --refinements 12 --inner-tol 1e-5

Runs `--repeat` solves of the k^-2 random-field workload at `--size`^3 unknowns with
the iteration cap `--maxit`, so that an ncu capture sees a handful of launches of
every kernel of the loop on fields larger than L2, and exits 0 whether or not the
cap stops the solve.  With --learned, the solver is flexible CG with the saved U-Net
as its coarse-grid correction (as in the benchmark's headline form); --cycle
F,C,RATIO selects the multigrid V-cycle with those smoother degrees.
"""
from __future__ import annotations

import argparse
import math

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
    ap.add_argument("--save-net", default=None, help="train the linear U-Net and save it here, then exit")
    ap.add_argument("--net-grid", type=int, default=16, help="edge of the network's grid")
    ap.add_argument("--coarsen", type=int, default=5, help="coarsenings whose coarsest-level operator --save-net learns")
    ap.add_argument("--learned", default=None, help="saved U-Net to use as the coarse-grid correction")
    ap.add_argument("--cycle", default=None, help="fine,coarse,ratio of the multigrid V-cycle (with --learned)")
    ap.add_argument("--inner-tol", type=float, default=3e-3)
    ap.add_argument("--post-smooth", action="store_true", help="Chebyshev post-smoothing on the solver's grid")
    ap.add_argument("--refinements", type=int, default=1)
    ap.add_argument("--krylov", default="bicgstab", choices=("bicgstab", "fcg"),
                    help="Krylov loop without --learned (fcg: flexible CG with the Chebyshev preconditioner)")
    a = ap.parse_args()
    if a.save_net:
        from parallelpoissonsolver_gb300 import learned
        train = learned.make_dataset(a.net_grid, range(10000, 10256), coarsen=a.coarsen)
        scale = learned.fit_scale(train)
        net = pps.UNet((16, 32, 64), seed=1, linear=True)
        learned.train(net, train, scale, 4000, lr=1e-3)
        net.save(a.save_net)
        import numpy as np
        with np.load(a.save_net) as d:
            np.savez(a.save_net, scale=np.array(scale), net_grid=np.array(a.net_grid), **{k: d[k] for k in d.files})
        print(f"saved {a.save_net}: scale {scale:.6g}")
        return
    grid = pps.BlockGrid.cube(a.size)
    b = workloads.random_field(a.size, seed=2)
    if a.learned:
        import numpy as np
        net = pps.UNet.load_file(a.learned)
        saved = np.load(a.learned)
        scale = float(saved["scale"])
        ng = int(saved["net_grid"]) if "net_grid" in saved.files else 32
        k = int(round(math.log2(a.size / ng)))
        gain = scale * ((2 ** k / (a.size + 1)) / (1.0 / (ng + 1))) ** 2
        s = pps.FlexibleCG(grid, pps.ChebyshevIteration(a.degree), tolerance=1e-10, max_iteration=a.maxit,
                           form=a.form, inner_maxit=a.maxit, max_refinements=a.refinements, use_graph=False,
                           inner_tol=a.inner_tol)
        flags = pps.LEARNED_PRECONDITIONER | pps.LEARNED_NO_FALLBACK
        if not a.cycle:
            flags |= pps.LEARNED_INITIAL_GUESS
        if a.post_smooth or not a.cycle:
            flags |= pps.LEARNED_POST_SMOOTH
        s.set_learned(net, k, gain, flags)
        if a.cycle:
            fd, cd, ratio = a.cycle.split(",")
            s.set_learned_cycle(int(fd), int(cd), float(ratio))
    else:
        cls = pps.FlexibleCG if a.krylov == "fcg" else pps.BiCGSTAB
        s = cls(grid, pps.ChebyshevIteration(a.degree), tolerance=1e-10, max_iteration=a.maxit,
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
