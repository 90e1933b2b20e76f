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


def test_batch_dataset_pairs_solve_the_level_operator():
    """make_dataset_batch: half unit-RMS random fields, half blob sums, each u the exact
    solution of the coarse-level operator for its b (checked on the CPU)."""
    n, k = 8, 2
    data = learned.make_dataset_batch(n, 7, 12, k, device="cpu", chunk=5)
    assert len(data) == 12
    h = 1.0 / (n + 1)
    t = learned.level_operator_1d(n, 2.0 ** (-k)) / (h * h)
    for i, (b, u) in enumerate(data):
        assert b.shape == (n, n, n) and u.shape == (n, n, n) and b.dtype == torch.float32
        bn, un = b.double().numpy(), u.double().numpy()
        au = (np.einsum("ai,ijk->ajk", t, un) + np.einsum("bj,ijk->ibk", t, un) + np.einsum("ck,ijk->ijc", t, un))
        assert np.abs(au - bn).max() < 1e-5 * np.abs(bn).max()
        if i < 6:
            assert abs(np.sqrt(np.mean(bn * bn)) - 1.0) < 1e-5   # random field, unit RMS
    # the same seed gives the same data
    again = learned.make_dataset_batch(n, 7, 12, k, device="cpu", chunk=5)
    assert all(torch.equal(a[0], c[0]) for a, c in zip(data, again))
