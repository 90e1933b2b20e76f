"""pps_solve on page-locked host arrays: copies overlapped with the solve.

On pinned arrays the MIXED Krylov solves upload b first and start on it as if x were
zero while x uploads on a second stream and a kernel tests it; a non-zero x restarts
the solve on it.  x is copied out after each refinement, the last copy overlapping
the final residual check.  Whatever x holds, the result must be bit for bit the one
of the same call on pageable arrays (copies before and after the solve), with the
same status, iteration count and residual history; pps_stats.copy_overlap records
which of the overlaps took place.
"""
import numpy as np
import pytest

import parallelpoissonsolver_gb300 as pps
from parallelpoissonsolver_gb300 import workloads

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

M = 48
UPLOAD, RESTART, DOWNLOAD = 1, 2, 4


def pinned_like(a):
    t = torch.empty(a.shape, dtype=torch.float64).pin_memory()
    out = t.numpy()
    out[...] = a
    return out


def make_solver(kind, tol=1e-10, maxit=2000, refinements=8):
    g = pps.BlockGrid.cube(M)
    if kind == "fcg":
        return pps.FlexibleCG(g, pps.ChebyshevIteration(11), tolerance=tol, max_iteration=maxit, form="mixed",
                              inner_tol=1e-5, max_refinements=refinements)
    return pps.BiCGSTAB(g, pps.ChebyshevIteration(11), tolerance=tol, max_iteration=maxit, form="mixed",
                        inner_tol=1e-5, max_refinements=refinements)


def run(s, x0, b0, pinned):
    x = pinned_like(x0) if pinned else x0.copy()
    b = pinned_like(b0) if pinned else b0.copy()
    st = s(x, b, raise_on_error=False)
    d = s.stats()
    return st, np.array(x), d, list(s.history())


def initial_guesses(b):
    shape = b.shape
    zero = np.zeros(shape)
    negzero = np.full(shape, -0.0)
    interior = np.zeros(shape)
    rng = np.random.default_rng(5)
    interior[2:-2, 2:-2, 2:-2] = 1e-3 * rng.standard_normal((M, M, M))   # the unknowns
    one_guard = np.zeros(shape)
    one_guard[0, 0, 0] = 1.0   # a guard corner: outside every stencil, still "non-zero"
    return {"zero": zero, "negzero": negzero, "interior": interior, "one_guard": one_guard}


@pytest.mark.parametrize("kind", ["fcg", "bicgstab"])
def test_pinned_solve_matches_pageable(gpu, kind):
    b0 = workloads.random_field(M, seed=71)
    s = make_solver(kind)
    for name, x0 in initial_guesses(b0).items():
        st_p, x_p, d_p, h_p = run(s, x0, b0, pinned=False)
        st_q, x_q, d_q, h_q = run(s, x0, b0, pinned=True)
        assert st_p == st_q == pps.OK, (name, st_p, st_q)
        assert np.array_equal(x_p.view(np.uint64), x_q.view(np.uint64)), name
        assert d_p["iterations"] == d_q["iterations"] and d_p["refinements"] == d_q["refinements"], name
        assert h_p == h_q, name
        assert d_p["copy_overlap"] == 0, name
        zero_x = name in ("zero", "negzero")
        expect = UPLOAD | DOWNLOAD | (0 if zero_x else RESTART)
        assert d_q["copy_overlap"] == expect, (name, d_q["copy_overlap"])
    s.close()


def test_pinned_solve_with_dirichlet_data(gpu):
    """Boundary values in x (the reference problem's exact solution on the faces): the
    first pass on x = 0 is void and the solve restarts on x."""
    s = make_solver("fcg")
    x0 = np.zeros(s.grid.shape)
    b0 = np.zeros(s.grid.shape)
    s.set_problem(x0, b0)
    assert np.any(x0 != 0)
    st_p, x_p, d_p, h_p = run(s, x0, b0, pinned=False)
    st_q, x_q, d_q, h_q = run(s, x0, b0, pinned=True)
    assert st_p == st_q == pps.OK
    assert np.array_equal(x_p.view(np.uint64), x_q.view(np.uint64))
    assert h_p == h_q
    assert d_q["copy_overlap"] == UPLOAD | RESTART | DOWNLOAD
    s.close()


def test_pinned_solve_already_converged(gpu):
    """x already meets the tolerance: no refinement, x comes back unchanged."""
    b0 = workloads.random_field(M, seed=72)
    s = make_solver("fcg")
    x_sol = np.zeros_like(b0)
    assert s(x_sol, b0.copy()) == pps.OK
    st_p, x_p, d_p, _ = run(s, x_sol, b0, pinned=False)
    st_q, x_q, d_q, _ = run(s, x_sol, b0, pinned=True)
    assert st_p == st_q == pps.OK
    assert d_q["refinements"] == 0
    assert np.array_equal(x_q.view(np.uint64), x_sol.view(np.uint64))
    assert np.array_equal(x_p.view(np.uint64), x_q.view(np.uint64))
    assert d_q["copy_overlap"] == UPLOAD | RESTART
    s.close()


def test_pinned_solve_not_converged_and_zero_rhs(gpu):
    b0 = workloads.random_field(M, seed=73)
    # one refinement of at most 3 iterations: PPS_NOT_CONVERGED, x still copied out
    s = make_solver("fcg", maxit=3, refinements=1)
    x0 = np.zeros_like(b0)
    st_p, x_p, _, _ = run(s, x0, b0, pinned=False)
    st_q, x_q, d_q, _ = run(s, x0, b0, pinned=True)
    assert st_p == st_q == pps.NOT_CONVERGED
    assert np.array_equal(x_p.view(np.uint64), x_q.view(np.uint64))
    assert np.any(x_q != 0)
    # b = 0 and x = 0: the zero right-hand side is reported on both paths
    zb = np.zeros_like(b0)
    st_p, _, _, _ = run(s, x0, zb, pinned=False)
    st_q, _, _, _ = run(s, x0, zb, pinned=True)
    assert st_p == st_q == pps.ERR_ZERO_RHS
    s.close()
