"""Batched solves in one persistent launch (no reference counterpart): flexible CG
with a multigrid V-cycle per problem, FP64 refinement, the whole solve one
cooperative kernel replayed as a CUDA graph.

* every problem of a batch of uneven cubes (edges 32-128, the batched workload's
  sizes) reaches the FP64 tolerance and agrees with the oracle's FP64 solution;
* two replays give bit-identical results (the per-problem sums are deterministic);
* a grid barrier whose wait limit runs out ends the solve with TIMEOUT, on the GPU,
  without a fault: the context stays usable and the next solve succeeds;
* grids the V-cycle cannot coarsen are rejected.
"""
import numpy as np
import pytest

import parallelpoissonsolver_gb300 as pps
from parallelpoissonsolver_gb300 import workloads
from conftest import rel_l2

pytestmark = pytest.mark.gpu

EDGES = [32, 48, 64, 96, 32, 128, 48]


def make(edges, seed0=70):
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
    oracle.solve(g, oracle.Config(tol=1e-13, maxit=20000, threads=8), x, b.copy())
    return x


def loaded(grids, fields, **kw):
    bt = pps.Batch(grids, tolerance=1e-10, inner_tol=1e-5, method="vcycle", **kw)
    for p, (x, b) in enumerate(fields):
        bt.set(p, x, b)
    return bt


def test_persistent_vcycle_batch_matches_oracle(gpu, oracle):
    grids, fields = make(EDGES)
    bt = loaded(grids, fields)
    assert bt.solve() == pps.OK, pps.last_error()
    st = bt.stats()
    assert st["converged"] == len(EDGES) and st["max_err_true"] <= 1e-10, st
    assert st["kernel_launches"] == 2 and st["graph_replays"] == 1
    for p, m in enumerate(EDGES):
        x, ps = bt.get(p)
        assert ps["err_true"] <= 1e-10 and ps["refinements"] >= 1
        assert ps["iterations"] <= 40, ps          # the V-cycle: about ten FCG iterations per refinement
        assert rel_l2(x, oracle_solution(oracle, m, fields[p][1])) < 1e-7
    bt.close()


def test_persistent_vcycle_batch_replays_bit_identically(gpu):
    grids, fields = make(EDGES[:4], seed0=90)
    bt = loaded(grids, fields)
    assert bt.solve() == pps.OK
    first = [bt.get(p)[0].copy() for p in range(len(grids))]
    for p, (x, b) in enumerate(fields):   # same inputs again: the graph is replayed
        bt.set(p, x, b)
    assert bt.solve() == pps.OK
    for p in range(len(grids)):
        assert np.array_equal(bt.get(p)[0], first[p])
    bt.close()


def test_barrier_wait_limit_runs_out_without_a_fault(gpu):
    grids, fields = make([32, 64, 32], seed0=110)
    bt = loaded(grids, fields)
    bt.set_wait_limit(1e-9)        # no barrier completes within a nanosecond
    assert bt.solve(raise_on_error=False) == pps.TIMEOUT
    assert "waited longer" in pps.last_error()
    bt.set_wait_limit(5.0)
    for p, (x, b) in enumerate(fields):
        bt.set(p, x, b)
    assert bt.solve() == pps.OK    # the context is intact
    assert bt.stats()["converged"] == 3
    bt.close()


def test_persistent_vcycle_batch_rejects_what_it_does_not_run(gpu):
    with pytest.raises(pps.PpsError):
        pps.Batch([pps.BlockGrid.cube(33)], method="vcycle")          # odd edge: no coarse level
    with pytest.raises(pps.PpsError):
        pps.Batch([pps.BlockGrid(npglobal=(34, 34, 66), ds=(1 / 33, 1 / 33, 1 / 65))], method="vcycle")
    with pytest.raises(pps.PpsError):
        pps.Batch([pps.BlockGrid.cube(32)]).set_wait_limit(1.0)       # the per-phase batch has no barrier
