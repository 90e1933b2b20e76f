"""Parity cases shared by the golden-fixture generator and the tests.

Each case is a single-rank problem of the reference solver: a grid, the solver
parameters (the reference's compile-time constants, solverSetup.hpp / inputParam.hpp)
and how its input fields are made:

  ("random", seed)  b ~ N(0,1) at the data nodes, random Dirichlet values on the
                    Dirichlet faces, random Neumann face data; numpy PCG64, so the
                    inputs are bit-identical on every machine.
  ("problem", p)    the built-in manufactured problem p (0 = the reference default
                    u = sin x + cos y + 3 sin z + x^2 y z + x^2 + 10, 1 = sine product);
                    its inputs are stored in the fixture because they go through libm.
  ("warm", seed)    a random problem whose x interior already holds a converged
                    solution, which exercises the reference's early return
                    (BiCGSTAB.hpp:118-122).

The compositions of inputParam.hpp beyond the default: krylov 2 is
ChebyshevIteration as the main solver (isMainLoop true, ALP/include/inputParam.hpp:37,
used with the eigenvalue rescaling set to 1 as its comment asks); precond 2 is a
BiCGSTAB object as the preconditioner (isMainLoop false, CPU/include/inputParam.hpp:30),
precond 3 a BaseCG object (inputParam.hpp:29), each with tolerance prec_tol, cap
prec_maxit and its own preconditioner prec_inner (0 none, 1 Chebyshev).  The CPU preset's inner tolerance is tollPreconditionerSolver *
tollScalingFactor = 1e4 * 1e-10, a hundred times the main one (solverSetup.hpp:22-33).

`store` = "full" keeps input and output fields; "summary" keeps iteration count,
residual history, checksums and a sample of the solution.
"""
from __future__ import annotations

import numpy as np

CPU = dict(krylov=0, precond=1, cheb_degree=11, cheb_eps=1e-4, rescale_min=500.0, rescale_max=1.0 - 1e-4,
           tol=1e-10, maxit=1700)


def cfg(**kw):
    c = dict(CPU)
    c.update(kw)
    return c


def cube(m):
    h = 1.0 / (m + 1)
    return dict(np=(m + 2,) * 3, ds=(h,) * 3, origin=(0.0, 0.0, 0.0))


CASES = [
    dict(name="dirichlet_random_m10", **cube(10), bcs=(0,) * 6, cfg=cfg(), inputs=("random", 1), store="full"),
    dict(name="dirichlet_problem0_aniso", np=(13, 11, 9), ds=(0.1, 0.12, 0.09), origin=(0.3, -0.2, 0.1),
         bcs=(0,) * 6, cfg=cfg(), inputs=("problem", 0), store="full"),
    dict(name="neumann_problem0_m10", **cube(10), bcs=(0, 1, 0, 1, 0, 1), cfg=cfg(), inputs=("problem", 0),
         store="full"),
    dict(name="neumann_random_ragged", np=(11, 10, 12), ds=(0.1, 0.1, 0.1), origin=(0.0, 0.0, 0.0),
         bcs=(1, 0, 0, 1, 1, 0), cfg=cfg(), inputs=("random", 2), store="full"),
    dict(name="alpaka_preset_m10", **cube(10), bcs=(0,) * 6,
         cfg=cfg(cheb_degree=24, cheb_eps=0.0, rescale_min=100.0, maxit=1000), inputs=("random", 3), store="full"),
    dict(name="cg_chebyshev_m10", **cube(10), bcs=(0,) * 6, cfg=cfg(krylov=1), inputs=("random", 4), store="full"),
    dict(name="cg_neumann_m8", **cube(8), bcs=(0, 1, 0, 1, 0, 1), cfg=cfg(krylov=1), inputs=("problem", 0),
         store="full"),
    dict(name="no_preconditioner_m10", **cube(10), bcs=(0,) * 6, cfg=cfg(precond=0), inputs=("random", 5),
         store="full"),
    dict(name="degree1_m8", **cube(8), bcs=(0,) * 6, cfg=cfg(cheb_degree=1), inputs=("random", 6), store="full"),
    dict(name="degree2_m8", **cube(8), bcs=(0,) * 6, cfg=cfg(cheb_degree=2), inputs=("random", 7), store="full"),
    dict(name="degree3_m8", **cube(8), bcs=(0,) * 6, cfg=cfg(cheb_degree=3), inputs=("random", 8), store="full"),
    dict(name="degree5_m9", **cube(9), bcs=(0, 0, 1, 0, 0, 0), cfg=cfg(cheb_degree=5), inputs=("random", 9),
         store="full"),
    dict(name="iteration_cap_m12", **cube(12), bcs=(0,) * 6, cfg=cfg(maxit=3), inputs=("random", 10), store="full"),
    dict(name="early_return_m8", **cube(8), bcs=(0,) * 6, cfg=cfg(), inputs=("warm", 11), store="full"),
    dict(name="single_unknown", np=(3, 3, 3), ds=(0.5, 0.5, 0.5), origin=(0.0, 0.0, 0.0), bcs=(0,) * 6,
         cfg=cfg(), inputs=("random", 12), store="full"),
    dict(name="thin_axis", np=(3, 9, 7), ds=(0.2, 0.1, 0.15), origin=(0.0, 0.0, 0.0), bcs=(0,) * 6, cfg=cfg(),
         inputs=("random", 13), store="full"),
    dict(name="tol1e13_m10", **cube(10), bcs=(0,) * 6, cfg=cfg(tol=1e-13, maxit=20000), inputs=("random", 14),
         store="full"),
    # 64^3 interior, h = 1/65: the sine right-hand side (an exact discrete eigenvector,
    # 1 iteration) and the non-degenerate companion (reference default manufactured solution).
    dict(name="sine_eigenvector_m64", **cube(64), bcs=(0,) * 6, cfg=cfg(), inputs=("problem", 1), store="summary"),
    dict(name="problem0_m64", **cube(64), bcs=(0,) * 6, cfg=cfg(), inputs=("problem", 0), store="summary"),
    dict(name="problem0_m64_tol1e13", **cube(64), bcs=(0,) * 6, cfg=cfg(tol=1e-13, maxit=20000),
         inputs=("problem", 0), store="summary"),
]

PREC_BICG = dict(precond=2, tol=1e-8, prec_tol=100.0 * 1e-8, prec_maxit=150, prec_inner=0)
CHEB_MAIN = dict(krylov=2, cheb_eps=0.0, rescale_min=1.0, rescale_max=1.0)

CASES += [
    dict(name="bicgstab_precond_m8", **cube(8), bcs=(0,) * 6, cfg=cfg(**PREC_BICG), inputs=("random", 20),
         store="full"),
    dict(name="bicgstab_precond_neumann_ragged", np=(9, 8, 10), ds=(0.1, 0.1, 0.1), origin=(0.0, 0.0, 0.0),
         bcs=(0, 1, 1, 0, 0, 1), cfg=cfg(**PREC_BICG), inputs=("random", 21), store="full"),
    dict(name="bicgstab_precond_cap3_m8", **cube(8), bcs=(0,) * 6, cfg=cfg(**{**PREC_BICG, "prec_maxit": 3}),
         inputs=("random", 22), store="full"),
    dict(name="bicgstab_precond_chebyshev_m8", **cube(8), bcs=(0,) * 6, cfg=cfg(**{**PREC_BICG, "prec_inner": 1}),
         inputs=("random", 23), store="full"),
    dict(name="cg_bicgstab_precond_m8", **cube(8), bcs=(0,) * 6, cfg=cfg(krylov=1, **PREC_BICG),
         inputs=("random", 24), store="full"),
    dict(name="bicgstab_precond_alpaka_m8", **cube(8), bcs=(0,) * 6,
         cfg=cfg(**{**PREC_BICG, "tol": 1e-10, "prec_tol": 1e8 * 1e-10, "prec_maxit": 500}), inputs=("random", 25),
         store="full"),
    dict(name="bicgstab_cg_precond_chebyshev_m8", **cube(8), bcs=(0,) * 6,
         cfg=cfg(**{**PREC_BICG, "precond": 3, "prec_inner": 1}), inputs=("random", 31), store="full"),
    dict(name="bicgstab_cg_precond_neumann_ragged", np=(9, 8, 10), ds=(0.1, 0.1, 0.1), origin=(0.0, 0.0, 0.0),
         bcs=(1, 0, 0, 1, 1, 0), cfg=cfg(**{**PREC_BICG, "precond": 3, "prec_inner": 1}), inputs=("random", 32),
         store="full"),
    dict(name="bicgstab_cg_precond_cap3_m8", **cube(8), bcs=(0,) * 6,
         cfg=cfg(**{**PREC_BICG, "precond": 3, "prec_inner": 1, "prec_maxit": 3}), inputs=("random", 33),
         store="full"),
    dict(name="chebyshev_main_d80_m8", **cube(8), bcs=(0,) * 6, cfg=cfg(cheb_degree=80, **CHEB_MAIN),
         inputs=("random", 26), store="full"),
    dict(name="chebyshev_main_d24_neumann_m8", **cube(8), bcs=(0, 1, 0, 1, 0, 1), cfg=cfg(cheb_degree=24, **CHEB_MAIN),
         inputs=("problem", 0), store="full"),
    dict(name="chebyshev_main_d1_m6", **cube(6), bcs=(0,) * 6, cfg=cfg(cheb_degree=1, **CHEB_MAIN),
         inputs=("random", 27), store="full"),
    dict(name="chebyshev_main_d2_m6", **cube(6), bcs=(0,) * 6, cfg=cfg(cheb_degree=2, **CHEB_MAIN),
         inputs=("random", 28), store="full"),
    dict(name="chebyshev_main_d3_m6", **cube(6), bcs=(0,) * 6, cfg=cfg(cheb_degree=3, **CHEB_MAIN),
         inputs=("random", 29), store="full"),
    dict(name="chebyshev_main_cpu_preset_m8", **cube(8), bcs=(0, 0, 1, 0, 0, 0), cfg=cfg(krylov=2, cheb_degree=11),
         inputs=("random", 30), store="full"),
]

BY_NAME = {c["name"]: c for c in CASES}


def shape(case):
    n = case["np"]
    return (n[2] + 2, n[1] + 2, n[0] + 2)


def face_shape(case, f):
    d = f // 2
    rest = [case["np"][a] for a in range(3) if a != d]
    return (rest[1], rest[0])


def random_inputs(case, seed):
    """x with random Dirichlet node values, b random at the data nodes, random Neumann faces."""
    rng = np.random.default_rng(seed)
    sh = shape(case)
    n = case["np"]
    b = np.zeros(sh)
    b[1:n[2] + 1, 1:n[1] + 1, 1:n[0] + 1] = rng.standard_normal((n[2], n[1], n[0]))
    x = np.zeros(sh)
    bnd = rng.standard_normal(sh)
    bcs = case["bcs"]
    # Dirichlet faces: the data-node plane of each face (applyDirichletBCsFromFunction's range)
    for f in range(6):
        if bcs[f] != 0:
            continue
        d, side = f // 2, f % 2
        sl = [slice(1, n[2] + 1), slice(1, n[1] + 1), slice(1, n[0] + 1)]
        axis = 2 - d
        sl[axis] = slice(1, 2) if side == 0 else slice(n[d], n[d] + 1)
        x[tuple(sl)] = bnd[tuple(sl)]
    faces = [rng.standard_normal(face_shape(case, f)) if bcs[f] == 1 else None for f in range(6)]
    return x, b, faces
