"""Flexible CG's direction kernel with its inputs staged in shared memory by TMA
(cp.async.bulk.tensor boxes from tiled tensor maps into a ring of planes, mbarrier
completion) against the kernel that loads them itself: the same tiles, per-point arithmetic and per-thread sums, so
whole MIXED solves must agree bit for bit (solution, iteration count, residual
history).  The grids cover a last x tile whose staged box runs past the row's end
(m = 128: 8 floats inside, the 512^3 case's shape; m = 252: 132 floats), a single tile
whose box starts before the row (m = 100), tile heights 2, 4 and 8 rows, and z chunks
of one to many planes."""
import numpy as np
import pytest

import parallelpoissonsolver_gb300 as pps
from parallelpoissonsolver_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,ty,waves", [(128, 8, 4), (128, 2, 1), (100, 4, 8), (252, 8, 2)])
def test_staged_direction_kernel_is_bit_identical(gpu, m, ty, waves):
    b = workloads.random_field(m, seed=40 + m)
    out = []
    for staged in (1, 0):
        s = pps.FlexibleCG(pps.BlockGrid.cube(m), pps.ChebyshevIteration(11), tolerance=1e-10, max_iteration=2000,
                           form="mixed", inner_tol=1e-5)
        t = s.tuning()
        assert t["fcg_staged"] == 0   # the default
        s.set_tuning({**t, "cheb_ty": ty, "cheb_cx": 4, "cheb_waves": waves, "fcg_staged": staged})
        x = np.zeros_like(b)
        assert s(x, b.copy()) == pps.OK
        out.append((x, s.get_num_iteration_final(), list(s.history()), s.get_error_compute_operator()))
        s.close()
    (xa, ia, ha, ea), (xb, ib, hb, eb) = out
    assert ea <= 1e-10
    assert ia == ib and ha == hb
    assert np.array_equal(xa.view(np.uint64), xb.view(np.uint64))
