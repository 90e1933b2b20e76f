"""The FP64 form against the reference's own solves of the 512^3 benchmark workload.

tests/golden/record_512.npz holds what the reference's BiCGSTAB + Chebyshev(11)
(solverPoissonMPI_CPU, compiled unchanged by `make -C oracle ref`) did on the 512^3
k^-2 random field (seed 2, Dirichlet 0), made by tests/golden/make_record_512.py:
iteration count, residual history and a 32,768-point sample of x at stop
tolerances 1e-10 and 1e-13, and the spread of the reference's own iteration count
and solution when b changes by one ulp in 1% of its entries.  The GPU regenerates
the field here; FFT libraries differ in the last bits, so its b matches the
record's to rounding, not bit for bit -- itself one more such perturbation.

Checked for the FP64 form:
* the first 10 residual-history entries agree to 1e-12 relative (the iterations
  have not yet amplified rounding differences);
* at 1e-10 the iteration count lies inside the reference's own spread (widened by
  one), and the sample lies as close to the record as the reference's perturbed
  solutions do (twice their largest distance);
* at 1e-13 the solutions agree to 1e-11 relative L2 on the sample.
"""
import os

import numpy as np
import pytest

import parallelpoissonsolver_gb300 as pps
from parallelpoissonsolver_gb300 import workloads

pytestmark = pytest.mark.gpu

RECORD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "record_512.npz")


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


def sample_rel(xs, ref):
    return float(np.linalg.norm(xs - ref) / np.linalg.norm(ref))


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
    ref_x = record["1em10_x_sample"]
    counts = [int(record["1em10_iterations"])] + [int(v) for v in record["spread_iterations"]]
    spread = max(sample_rel(xs, ref_x) for xs in record["spread_x_sample"])
    rel = sample_rel(x.ravel()[idx], ref_x)
    print(f"\n512^3 tol 1e-10: FP64 form {it} iterations; the reference {counts[0]}, perturbed {counts[1:]}; "
          f"sample rel-L2 {rel:.3e} (reference perturbed: up to {spread:.3e}); true residual {err:.3e}")
    assert err <= 1e-10
    h = np.asarray(hist)[:11]
    ref_h = record["1em10_history"][:11]
    assert np.max(np.abs(h - ref_h) / ref_h) <= 1e-12
    assert min(counts) - 1 <= it <= max(counts) + 1, (it, counts)
    assert rel <= 2.0 * spread, (rel, spread)


def test_fp64_512_tol1e13_against_reference(gpu, record, workload):
    m, b0, idx = workload
    x, it, hist, err = solve_fp64(m, b0, 1e-13)
    rel = sample_rel(x.ravel()[idx], record["1em13_x_sample"])
    print(f"\n512^3 tol 1e-13: FP64 form {it} iterations, reference {int(record['1em13_iterations'])}; "
          f"sample rel-L2 {rel:.3e}; true residual {err:.3e} (reference {float(record['1em13_err_true']):.3e})")
    # at 1e-13 the true residual sits at the FP64 floor of the normalised system
    assert err <= 10.0 * float(record["1em13_err_true"])
    assert rel <= 1e-11
