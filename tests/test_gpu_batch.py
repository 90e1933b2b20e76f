"""Batched solves (no reference counterpart): every problem of a batch of uneven
grids reaches the FP64 tolerance and agrees with the oracle's FP64 solution of the
same problem; graph replay and direct launches give the same iterates; the
autotuner's tiles keep the results."""
import numpy as np
import pytest

import parallelpoissonsolver_gb300 as pps
from parallelpoissonsolver_gb300 import workloads
from conftest import rel_l2

pytestmark = pytest.mark.gpu

EDGES = [12, 20, 9, 16, 24, 12, 31]


def make(edges, seed0=40):
    grids = [pps.BlockGrid.cube(m) for m in edges]
    fields = []
    for i, m in enumerate(edges):
        b = workloads.blobs(m, seed0 + i)
        if not np.any(b):
            b[2:-2, 2:-2, 2:-2] = 1.0
        fields.append((np.zeros_like(b), b))
    return grids, fields


def oracle_solution(oracle, m, b):
    g = oracle.cube(m)
    x = np.zeros_like(b)
    oracle.solve(g, oracle.Config(tol=1e-13, maxit=20000), x, b.copy())
    return x


@pytest.mark.parametrize("graph", [True, False])
def test_batch_matches_oracle(gpu, oracle, graph):
    grids, fields = make(EDGES)
    bt = pps.Batch(grids, tolerance=1e-10, use_graph=graph)
    for p, (x, b) in enumerate(fields):
        bt.set(p, x, b)
    assert bt.solve() == pps.OK
    st = bt.stats()
    assert st["converged"] == len(EDGES) and st["max_err_true"] <= 1e-10
    for p, m in enumerate(EDGES):
        x, ps = bt.get(p)
        assert ps["err_true"] <= 1e-10 and ps["refinements"] >= 1
        assert rel_l2(x, oracle_solution(oracle, m, fields[p][1])) < 1e-6
    bt.close()


def test_batch_graph_equals_direct_and_autotune(gpu):
    grids, fields = make(EDGES[:4], seed0=60)
    outs = []
    for graph, tune in [(True, False), (False, False), (True, True)]:
        bt = pps.Batch(grids, use_graph=graph)
        if tune:
            tiles = bt.autotune()
            assert all(cx in (1, 2, 4) and kc in (8, 16, 32, 64, 128) for cx, kc in tiles)
        for p, (x, b) in enumerate(fields):
            bt.set(p, x, b)
        assert bt.solve() == pps.OK
        outs.append([bt.get(p)[0] for p in range(len(grids))])
        bt.close()
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)          # same launches, same order: identical bits
    for a, b in zip(outs[0], outs[2]):
        assert rel_l2(a, b) < 1e-8           # other tiles: other rounding, same solution


def test_batch_rejects_what_it_does_not_run(gpu):
    with pytest.raises(pps.PpsError):
        pps.Batch([pps.BlockGrid.cube(8, bcs=(0, 1, 0, 0, 0, 0))])
    with pytest.raises(pps.PpsError):
        pps.Batch([pps.BlockGrid.cube(8)], preconditioner=pps.ChebyshevIteration(3))
