"""pps_apply_operator_noalloc: the operator apply for callers that cannot allocate
device memory (allocation-free loops, plugins whose host owns all device memory,
fixed memory budgets).  Called through the C ABI on device buffers the test owns,
twice in a row, and checked against the existing entry point pps_apply_operator
(FP64 form) and against the oracle's operator (the reference's
MatrixFreeOperatorA, matrixFreeOperatorA.hpp:22-39) with the tolerance of the
operator-kernel test (1e-12 of the largest value), and its energy sum u.(Au)
against the same sum taken on the host.  Overlapping buffers are rejected.

This file is named to be collected last, so a run that stops at the first failure
has already run every other test."""
import numpy as np
import pytest

import parallelpoissonsolver_gb300 as pps

pytestmark = pytest.mark.gpu


def test_noalloc_operator_matches_existing_entry_point(gpu, oracle):
    torch = pytest.importorskip("torch")
    grid = pps.BlockGrid(npglobal=(37, 29, 41), ds=(0.05, 0.07, 0.04), bcs=(0, 1, 1, 0, 0, 0))
    og = oracle.Grid(np=grid.npglobal, ds=grid.ds, bcs=grid.bcs)
    sl = grid.unknowns()
    solver = pps.BiCGSTAB(grid, pps.ChebyshevIteration(11), form="fp64")
    rng = np.random.default_rng(2024)
    energy = torch.zeros(1, dtype=torch.float64, device="cuda")
    for call in range(2):
        u = rng.standard_normal(grid.shape)
        fill = rng.standard_normal(grid.shape)       # entries outside the unknowns must survive
        want = solver.apply_operator(u, fill.copy())
        u_d = torch.from_numpy(u).cuda()
        out_d = torch.from_numpy(fill.copy()).cuda()
        torch.cuda.synchronize()
        st = pps.apply_operator_noalloc(grid, u_d.data_ptr(), out_d.data_ptr(), energy.data_ptr(),
                                        torch.cuda.current_stream().cuda_stream)
        assert st == pps.OK, pps.last_error()
        torch.cuda.synchronize()
        got = out_d.cpu().numpy()
        scale = np.max(np.abs(want[sl]))
        assert np.max(np.abs(got[sl] - want[sl])) <= 1e-12 * scale, f"call {call}"
        ref = oracle.apply_A(og, u)
        assert np.max(np.abs(got[sl] - ref[sl])) <= 1e-12 * np.max(np.abs(ref[sl])), f"call {call}: vs the oracle"
        mask = np.ones(grid.shape, bool)
        mask[sl] = False
        assert np.array_equal(got[mask], fill[mask]), f"call {call}: entries outside the unknowns changed"
        e_host = float(np.sum(u[sl] * want[sl]))
        assert abs(energy.item() - e_host) <= 1e-12 * np.sum(np.abs(u[sl] * want[sl])), f"call {call}"
    solver.close()


def test_noalloc_rejects_grids_beyond_the_scratch(gpu):
    torch = pytest.importorskip("torch")
    # 4096 x 4096 planes need 128 x 512 tiles = 65536 blocks of partials (> 16384)
    grid = pps.BlockGrid(npglobal=(4098, 4098, 3), ds=(1e-3, 1e-3, 1e-3))
    dummy = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = pps.apply_operator_noalloc(grid, dummy.data_ptr(), dummy.data_ptr(), dummy.data_ptr(), 0)
    assert st == pps.ERR_INVALID_ARG
    assert "static scratch" in pps.last_error()


def test_noalloc_rejects_overlapping_buffers(gpu):
    torch = pytest.importorskip("torch")
    grid = pps.BlockGrid.cube(6)
    u = torch.zeros(grid.shape, dtype=torch.float64, device="cuda")
    e = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = pps.apply_operator_noalloc(grid, u.data_ptr(), u.data_ptr(), e.data_ptr(), 0)
    assert st == pps.ERR_INVALID_ARG and "overlap" in pps.last_error()
    o = torch.zeros(grid.shape, dtype=torch.float64, device="cuda")
    st = pps.apply_operator_noalloc(grid, u.data_ptr(), o.data_ptr(), u.data_ptr() + 8, 0)   # energy inside u
    assert st == pps.ERR_INVALID_ARG and "overlap" in pps.last_error()
