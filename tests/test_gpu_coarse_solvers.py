"""What the trained network earns inside the learned multigrid V-cycle.

The same flexible CG + V-cycle (Chebyshev(5) on the solver's grid, Jacobi-scaled
Chebyshev(4) on the coarse levels, ratio 8) is run with its coarsest level (16^3)
solved four ways (pps_set_coarse_solver): the network trained on that level's
operator, no correction, the coarse smoother, and the level operator's exact
inverse.  The fallback is off, so each cycle's own convergence shows.

The network must do the exact solve's job (within one iteration of it) and cut the
iterations of the cycle without it (no correction, or smoothing only) at least in
half.  At 128^3 on a k^-2 field this measured 10 (network), 10 (exact), 36 (smooth)
and 59 (none) iterations.
"""
import math

import numpy as np
import pytest

import parallelpoissonsolver_gb300 as pps
from parallelpoissonsolver_gb300 import learned, workloads

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

NET_GRID = 16


@pytest.fixture(scope="module")
def coarse_net(gpu):
    m = 128
    k = int(round(math.log2(m / NET_GRID)))
    train = learned.make_dataset_batch(NET_GRID, 10000, 4000, k, device=0)
    scale = learned.fit_scale(train)
    net = pps.UNet((16, 32, 64), seed=1, linear=True)
    learned.train(net, train, scale, 4000, lr=1e-3)
    gain = scale * ((2 ** k / (m + 1)) / (1.0 / (NET_GRID + 1))) ** 2
    yield net, k, gain
    net.close()


def test_network_against_the_plain_coarse_solvers(coarse_net):
    net, k, gain = coarse_net
    m = 128
    b = workloads.random_field(m, seed=30042)
    s = pps.FlexibleCG(pps.BlockGrid.cube(m), pps.ChebyshevIteration(11), tolerance=1e-10, max_iteration=2000,
                       form="mixed", inner_tol=1e-5)
    s.set_learned(net, k, gain, pps.LEARNED_PRECONDITIONER | pps.LEARNED_NO_FALLBACK)
    s.set_learned_cycle(5, 4, 8.0)
    its = {}
    for name, kind in (("network", pps.COARSE_NETWORK), ("zero", pps.COARSE_ZERO), ("smooth", pps.COARSE_SMOOTH),
                       ("exact", pps.COARSE_EXACT)):
        s.set_coarse_solver(kind)
        x = np.zeros_like(b)
        assert s(x, b.copy()) == pps.OK, name
        assert s.get_error_compute_operator() <= 1e-10, name
        its[name] = s.get_num_iteration_final()
    s.close()
    print("\n128^3 V-cycle iterations by coarsest-level solver:", its)
    assert its["network"] <= its["exact"] + 1, its
    assert 2 * its["network"] <= its["zero"], its
    assert 2 * its["network"] <= its["smooth"], its


def test_coarse_solver_choice_is_validated(gpu):
    s = pps.FlexibleCG(pps.BlockGrid.cube(64), pps.ChebyshevIteration(11), form="mixed")
    with pytest.raises(pps.PpsError):
        s.set_coarse_solver(pps.COARSE_EXACT)          # no network attached: no cycle to put it in
    net = pps.UNet((16, 32, 64), seed=2, linear=True)
    s.set_learned(net, 2, 1.0, pps.LEARNED_PRECONDITIONER)
    s.set_learned_cycle(5, 0, 8.0)
    with pytest.raises(pps.PpsError):
        s.set_coarse_solver(pps.COARSE_SMOOTH)         # the coarse levels have no smoother (degree 0)
    with pytest.raises(pps.PpsError):
        s.set_coarse_solver(7)
    s.set_coarse_solver(pps.COARSE_EXACT)
    s.close()
    net.close()
