"""Host-side pieces of the learned preconditioner's training pipeline (no GPU): the
coarse-level operator and its exact tensor-product solve that make the training
targets for the multigrid cycle's coarsest level."""
import numpy as np
import pytest

from parallelpoissonsolver_gb300 import learned

torch = pytest.importorskip("torch")


def test_level_operator_is_the_uniform_second_difference_at_gap_one():
    t = learned.level_operator_1d(7, 1.0)
    want = np.diag(-2.0 * np.ones(7)) + np.diag(np.ones(6), 1) + np.diag(np.ones(6), -1)
    assert np.array_equal(t, want)


def test_level_operator_matches_the_unequal_spacing_formula():
    # u'' at the last unknown with neighbours at distance 1 (below) and gap (the wall, u = 0)
    gap = 0.125
    t = learned.level_operator_1d(5, gap)
    x = np.arange(1, 6, dtype=float)
    wall = 5.0 + gap
    u = (x - 0.0) * (wall - x)          # quadratic vanishing on both walls: u'' = -2
    assert np.allclose((t @ u)[-1], -2.0)
    assert np.allclose((t @ u)[1:-1], -2.0)


@pytest.mark.parametrize("gap", [1.0, 0.25, 1.0 / 16])
def test_level_solve_is_exact(gap):
    n, h = 10, 0.1
    rng = np.random.default_rng(3)
    b = rng.standard_normal((n, n, n))
    u = learned.level_solve(torch.from_numpy(b), h, gap).numpy()
    t = learned.level_operator_1d(n, gap) / (h * h)
    au = (np.einsum("ai,ijk->ajk", t, u) + np.einsum("bj,ijk->ibk", t, u) + np.einsum("ck,ijk->ijc", t, u))
    assert np.abs(au - b).max() < 1e-10 * np.abs(b).max()
