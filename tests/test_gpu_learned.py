"""The learned preconditioner end to end (no reference counterpart): a linear U-Net
trained on the GPU by the library's own kernels on 32^3 (f, u) pairs solved by the
plain FP64 solver, used as the coarse-grid solver inside flexible CG; it must cut the
iteration count of the method without it and still meet the FP64 tolerance, and an
untrained network must trigger the fallback to the plain preconditioner."""
import math

import numpy as np
import pytest

import parallelpoissonsolver_gb300 as pps
from parallelpoissonsolver_gb300 import learned
from conftest import rel_l2

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

FLAGS = pps.LEARNED_INITIAL_GUESS | pps.LEARNED_PRECONDITIONER | pps.LEARNED_POST_SMOOTH


@pytest.fixture(scope="module")
def trained(gpu):
    train = learned.make_dataset(32, range(10000, 10128))
    held = learned.make_dataset(32, range(30000, 30004))
    scale = learned.fit_scale(train)
    net = pps.UNet((16, 32, 64), seed=1, linear=True)
    losses = learned.train(net, train, scale, 2500, lr=1e-3)
    errs = learned.evaluate(net, held, scale)
    yield net, scale, losses, errs
    net.close()


def gain_for(m, scale):
    k = int(round(math.log2(m / 32)))
    return k, scale * ((2 ** k / (m + 1)) / (1.0 / 33)) ** 2


def test_training_reaches_a_useful_network(trained):
    net, scale, losses, errs = trained
    assert np.mean(losses[-100:]) < 0.1 * np.mean(losses[:100])
    assert max(errs) < 0.15, errs


@pytest.mark.parametrize("form", ["fp64", "mixed"])
def test_learned_preconditioner_cuts_iterations(trained, oracle, form):
    net, scale, _, _ = trained
    m = 64
    grid = pps.BlockGrid.cube(m)
    k, gain = gain_for(m, scale)
    b = learned.rhs(m, 30010, "field")
    x_ref = np.zeros_like(b)
    oracle.solve(oracle.cube(m), oracle.Config(tol=1e-13, maxit=20000, threads=4), x_ref, b.copy())
    plain = pps.FlexibleCG(grid, pps.ChebyshevIteration(11), tolerance=1e-10, form=form)
    x0 = np.zeros_like(b)
    assert plain(x0, b.copy()) == pps.OK
    it_plain = plain.get_num_iteration_final()
    s = pps.FlexibleCG(grid, pps.ChebyshevIteration(11), tolerance=1e-10, form=form, use_graph=False)
    s.set_learned(net, k, gain, FLAGS)
    x = np.zeros_like(b)
    assert s(x, b.copy()) == pps.OK
    st = s.stats()
    assert st["fallback_iteration"] == -1 and st["learned_applications"] > 0
    assert s.get_error_compute_operator() <= 1e-10
    assert s.get_num_iteration_final() <= 0.5 * it_plain, (s.get_num_iteration_final(), it_plain)
    assert rel_l2(x, x_ref) < 1e-6


def test_untrained_network_falls_back(gpu, oracle):
    net = pps.UNet((16, 32, 64), seed=5)                 # random weights
    m = 64
    grid = pps.BlockGrid.cube(m)
    b = learned.rhs(m, 30011, "blobs")
    s = pps.FlexibleCG(grid, pps.ChebyshevIteration(11), tolerance=1e-10, form="fp64", use_graph=False)
    s.set_learned(net, 1, 1e-3, pps.LEARNED_PRECONDITIONER)
    x = np.zeros_like(b)
    assert s(x, b.copy()) == pps.OK
    assert s.stats()["fallback_iteration"] >= 4
    assert s.get_error_compute_operator() <= 1e-10
    net.close()


def test_set_learned_rejects_unsupported(gpu):
    net = pps.UNet((16, 32, 64), seed=5)
    with pytest.raises(pps.PpsError):
        pps.FlexibleCG(pps.BlockGrid.cube(30), form="fp64").set_learned(net, 0, 1.0, FLAGS)   # 30 % 4 != 0
    with pytest.raises(pps.PpsError):
        pps.BiCGSTAB(pps.BlockGrid.cube(32), form="parity").set_learned(net, 0, 1.0, FLAGS)
    net.close()
