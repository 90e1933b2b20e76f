"""The FP64 form against the reference's own solve of the 512^3 benchmark workload.

tests/golden/record_512.npz holds what the reference's BiCGSTAB + Chebyshev(11)
(solverPoissonMPI_CPU, compiled unchanged by `make -C oracle ref`) did on the
512^3 k^-2 random field (seed 2, Dirichlet 0): iteration count, residual history
and a 32,768-point sample of x, at stop tolerances 1e-10 and 1e-13
(tests/golden/make_record_512.py made it).  The GPU regenerates the same field
here; FFT libraries differ in the last bits, so its b matches the record's to
rounding, not bit for bit.

Checked:
* the first 10 residual-history entries agree to 1e-12 relative (the iterations
  have not yet amplified rounding differences);
* at 1e-13 the solutions agree to 1e-11 relative L2 on the sample;
* at 1e-10 the iteration count is within ITER_BAND of the reference's and the
  sample agrees to 1e-8 (two solutions stopped at 1e-10 differ by what the stop
  leaves unsolved: the reference rebuilt with reassociated sums differs from
  itself by 2.8e-11 at 64^3, and the difference grows with the iteration count).
"""
import os

import numpy as np
import pytest

import parallelpoissonsolver_gb300 as pps
from parallelpoissonsolver_gb300 import workloads

pytestmark = pytest.mark.gpu

RECORD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "record_512.npz")
# BiCGSTAB amplifies rounding differences (the histories decorrelate after about 30
# iterations), so no implementation that sums in another order can promise the
# reference's count; this is the band the FP64 form holds on this workload.
ITER_BAND = 1


@pytest.fixture(scope="module")
def record():
    return dict(np.load(RECORD))


@pytest.fixture(scope="module")
def workload(record):
    m = int(record["m"])
    b = workloads.random_field(m, seed=2)
    idx = record["sample_index"]
    assert np.max(np.abs(b.ravel()[idx] - record["b_sample"])) <= 1e-12 * np.max(np.abs(record["b_sample"]))
    assert abs(np.sqrt((b * b).sum()) / record["b_l2"] - 1.0) <= 1e-12
    return m, b, idx


def sample_rel(x, idx, ref):
    d = x.ravel()[idx] - ref
    return float(np.linalg.norm(d) / np.linalg.norm(ref))


def solve_fp64(m, b0, tol):
    g = pps.BlockGrid.cube(m)
    s = pps.BiCGSTAB(g, pps.ChebyshevIteration(11), tolerance=tol, max_iteration=1700, form="fp64")
    x, b = np.zeros_like(b0), b0.copy()
    assert s(x, b) == pps.OK
    out = (x, s.get_num_iteration_final(), s.history(), s.get_error_compute_operator())
    s.close()
    return out


def test_fp64_512_tol1e10_against_reference(gpu, record, workload):
    m, b0, idx = workload
    x, it, hist, err = solve_fp64(m, b0, 1e-10)
    ref_it = int(record["1em10_iterations"])
    ref_h = record["1em10_history"]
    print(f"\n512^3 tol 1e-10: FP64 form {it} iterations, reference {ref_it}; "
          f"sample rel-L2 {sample_rel(x, idx, record['1em10_x_sample']):.3e}; true residual {err:.3e}")
    assert err <= 1e-10
    h = np.asarray(hist)[:11]
    assert np.max(np.abs(h - ref_h[:11]) / ref_h[:11]) <= 1e-12
    assert abs(it - ref_it) <= ITER_BAND
    assert sample_rel(x, idx, record["1em10_x_sample"]) <= 1e-8


def test_fp64_512_tol1e13_against_reference(gpu, record, workload):
    m, b0, idx = workload
    x, it, hist, err = solve_fp64(m, b0, 1e-13)
    rel = sample_rel(x, idx, record["1em13_x_sample"])
    print(f"\n512^3 tol 1e-13: FP64 form {it} iterations, reference {int(record['1em13_iterations'])}; "
          f"sample rel-L2 {rel:.3e}")
    assert err <= 1e-13
    assert rel <= 1e-11
