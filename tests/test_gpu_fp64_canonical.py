"""The FP64 form's results depend on the grid and the data alone.

Its sums (BiCGSTAB's and CG's dots, the start residual, ||b_adj||, the final true
residual) are canonical: one partial per fixed cell of the grid (32 columns of a row
over a z chunk fixed by the grid), summed by a fixed tree.  So every tiling the
autotuner may choose gives bit-identical iterates, iteration counts and residual
histories.  Without it the block partials followed the tile shape and the 512^3
iteration count moved between 159 and 167 from one tuning to the next.
"""
import numpy as np
import pytest

import parallelpoissonsolver_gb300 as pps
from cases import BY_NAME
from conftest import load_golden, rel_l2, same_bits

pytestmark = pytest.mark.gpu

TUNINGS = [
    dict(cheb_ty=8, cheb_cx=1, cheb_waves=4, other_ty=8, other_waves=4),
    dict(cheb_ty=2, cheb_cx=2, cheb_waves=1, other_ty=4, other_waves=8),
    dict(cheb_ty=4, cheb_cx=1, cheb_waves=8, other_ty=2, other_waves=1),
]


def tuned(solver, t):
    solver.set_tuning({**solver.tuning(), **t})
    return solver


def random_cube(m, seed):
    rng = np.random.default_rng(seed)
    g = pps.BlockGrid.cube(m)
    b = g.new_field()
    b[g.unknowns()] = rng.standard_normal((m, m, m))
    return g, b


@pytest.mark.parametrize("krylov", ["bicgstab", "cg"])
def test_fp64_form_is_tile_independent(gpu, oracle, krylov):
    m = 48
    g, b0 = random_cube(m, 17)
    cls = pps.BiCGSTAB if krylov == "bicgstab" else pps.BaseCG
    runs = []
    for t in TUNINGS:
        s = tuned(cls(g, pps.ChebyshevIteration(11), tolerance=1e-10, max_iteration=1700, form="fp64"), t)
        x, b = g.new_field(), b0.copy()
        assert s(x, b) == pps.OK
        runs.append((x, s.get_num_iteration_final(), s.history(), s.get_error_compute_operator()))
        s.close()
    x0, it0, h0, e0 = runs[0]
    for x, it, h, e in runs[1:]:
        assert it == it0
        assert same_bits(h, h0)
        assert same_bits(x, x0)
        assert same_bits([e], [e0])
    # Against the reference: on white noise BiCGSTAB's count is chaotic in rounding.
    # The reference's own count (the oracle is bit-identical to it) moves by several
    # iterations when b changes by one ulp in 1% of its entries (39..43 here), and its
    # solutions then differ by 5e-9..7e-9 relative L2 at the 1e-10 stop.  The FP64
    # form, which rounds differently, must land inside that spread.
    og = oracle.cube(m)
    cfg = oracle.Config(krylov=0 if krylov == "bicgstab" else 1, tol=1e-10, threads=4)
    counts, sols = [], []
    for trial in range(6):
        bo = b0.copy()
        if trial:
            mask = np.random.default_rng(trial).random(bo.shape) < 0.01
            bo[mask] = np.nextafter(bo[mask], np.inf)
        xo = np.zeros_like(b0)
        counts.append(oracle.solve(og, cfg, xo, bo).iterations)
        sols.append(xo)
    spread = max(rel_l2(x, sols[0]) for x in sols[1:])
    assert min(counts) - 1 <= it0 <= max(counts) + 1, (it0, counts)
    assert rel_l2(x0, sols[0]) <= max(2.0 * spread, 1e-9), (rel_l2(x0, sols[0]), spread)


def test_fp64_neumann_ragged_is_tile_independent(gpu, oracle):
    case = BY_NAME["neumann_random_ragged"]
    gold = load_golden(case["name"])
    faces = [gold.get(f"face{f}") for f in range(6)]
    grid = pps.BlockGrid(npglobal=case["np"], ds=case["ds"], origin=case["origin"], bcs=case["bcs"])
    c = case["cfg"]
    outs = []
    for t in TUNINGS:
        s = tuned(pps.BiCGSTAB(grid, pps.ChebyshevIteration(c["cheb_degree"], c["cheb_eps"], c["rescale_min"]),
                               tolerance=c["tol"], max_iteration=c["maxit"], form="fp64"), t)
        for f, a in enumerate(faces):
            if a is not None:
                s.set_neumann(f, a)
        x, b = gold["x_in"].copy(), gold["b_in"].copy()
        assert s(x, b) == pps.OK
        outs.append((x, s.get_num_iteration_final(), s.history()))
        s.close()
    for x, it, h in outs[1:]:
        assert it == outs[0][1] and same_bits(h, outs[0][2]) and same_bits(x, outs[0][0])
    assert abs(outs[0][1] - int(gold["iterations"])) <= 1
