"""Every form reaches the FP64 tolerance and shows the scheme's second-order
discretisation error on a manufactured solution: u = sin(pi x) sin(pi y) sin(pi z) on
the unit cube with homogeneous Dirichlet boundaries, b = A u = -3 pi^2 u (A the
positive-sign 7-point Laplacian of the reference), solved on m = 16/32/64 (32/64/128 for
the learned V-cycle) unknowns per axis; the max error against the exact u must fall as
h^2."""
import math

import numpy as np
import pytest

import parallelpoissonsolver_gb300 as pps
from parallelpoissonsolver_gb300 import learned

pytestmark = pytest.mark.gpu


def sine_problem(m):
    grid = pps.BlockGrid.cube(m)
    h = 1.0 / (m + 1)
    c = np.arange(0, m + 2) * h            # data nodes 0..m+1 (the boundary nodes are 0 and m+1)
    u1 = np.sin(np.pi * c)
    u = u1[:, None, None] * u1[None, :, None] * u1[None, None, :]
    x = grid.new_field()
    b = grid.new_field()
    b[1:m + 3, 1:m + 3, 1:m + 3] = -3.0 * np.pi ** 2 * u
    b[0, :, :] = b[-1, :, :] = 0.0
    inner = (slice(2, m + 2),) * 3
    bb = np.zeros_like(b)
    bb[inner] = b[inner]
    return grid, x, bb, u


def observed_order(ms, errs):
    hs = [1.0 / (m + 1) for m in ms]
    return [math.log(errs[i] / errs[i + 1]) / math.log(hs[i] / hs[i + 1]) for i in range(len(ms) - 1)]


def solve_and_error(s, grid, x, b, u, m):
    st = s(x, b)
    assert st == pps.OK, pps.status_string(st)
    assert s.get_error_compute_operator() <= 1e-10
    return float(np.max(np.abs(x[1:m + 3, 1:m + 3, 1:m + 3] - u)))


@pytest.mark.parametrize("form", ["parity", "fp64", "mixed"])
def test_second_order_reference_method(gpu, form):
    ms = (16, 32) if form == "parity" else (16, 32, 64)
    errs = []
    for m in ms:
        grid, x, b, u = sine_problem(m)
        s = pps.BiCGSTAB(grid, pps.ChebyshevIteration(11), tolerance=1e-10, max_iteration=5000, form=form)
        errs.append(solve_and_error(s, grid, x, b, u, m))
        s.close()
    for p in observed_order(ms, errs):
        assert 1.9 < p < 2.1, (errs, observed_order(ms, errs))


def test_second_order_learned_vcycle(gpu):
    ms = (32, 64, 128)
    errs = []
    for m in ms:
        k = int(round(math.log2(m / 16)))
        train = learned.make_dataset(16, range(10000, 10032), coarsen=k)
        scale = learned.fit_scale(train)
        net = pps.UNet((16, 32, 64), seed=1, linear=True)
        learned.train(net, train, scale, 300, lr=1e-3)
        gain = scale * ((2 ** k / (m + 1)) / (1.0 / 17)) ** 2
        grid, x, b, u = sine_problem(m)
        s = pps.FlexibleCG(grid, pps.ChebyshevIteration(11), tolerance=1e-10, form="mixed", inner_tol=1e-5)
        s.set_learned(net, k, gain, pps.LEARNED_PRECONDITIONER)
        s.set_learned_cycle(5, 4, 8.0)
        errs.append(solve_and_error(s, grid, x, b, u, m))
        assert s.stats()["learned_applications"] > 0
        s.close()
        net.close()
    for p in observed_order(ms, errs):
        assert 1.9 < p < 2.1, (errs, observed_order(ms, errs))
