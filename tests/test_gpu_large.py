"""The 1024^3 path (the charges workload: 64 Gaussian charges on a k^-3 background,
8.6 GB per FP64 field) runs end to end on the GPU at a capped iteration count: the
mixed flexible CG with the learned V-cycle over seven levels (the network on the
16^3 level) and the plain FP64 BiCGSTAB + Chebyshev.  Both must reduce the residual
without a CUDA error; the full solves to 1e-10 are timed by bench.py."""
import math

import numpy as np
import pytest

import parallelpoissonsolver_gb300 as pps
from parallelpoissonsolver_gb300 import learned, workloads

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_1024_mixed_learned_and_plain_fp64_capped(gpu):
    m = 1024
    grid = pps.BlockGrid.cube(m)
    b = workloads.charges_device(m, device="cuda:0")
    x = torch.zeros_like(b)
    k = int(round(math.log2(m / 16)))
    train = learned.make_dataset_batch(16, 10000, 512, k, device=0)
    scale = learned.fit_scale(train)
    net = pps.UNet((16, 32, 64), seed=1, linear=True)
    learned.train(net, train, scale, 500, lr=1e-3)
    gain = scale * ((2 ** k / (m + 1)) / (1.0 / 17)) ** 2
    s = pps.FlexibleCG(grid, pps.ChebyshevIteration(11), tolerance=1e-10, max_iteration=4, form="mixed",
                       inner_tol=1e-5, inner_maxit=4, max_refinements=1)
    s.set_learned(net, k, gain, pps.LEARNED_PRECONDITIONER | pps.LEARNED_NO_FALLBACK)
    s.set_learned_cycle(5, 4, 8.0)
    torch.cuda.synchronize()
    st = s.solve_device(x.data_ptr(), b.data_ptr(), raise_on_error=False)
    assert st in (pps.OK, pps.NOT_CONVERGED), pps.status_string(st)
    d = s.stats()
    assert d["learned_applications"] > 0 and d["iterations"] >= 1
    assert np.isfinite(d["err_true"]) and d["err_true"] < 0.1, d["err_true"]
    s.close()
    net.close()
    x.zero_()
    p = pps.BiCGSTAB(grid, pps.ChebyshevIteration(11), tolerance=1e-10, max_iteration=2, form="fp64")
    torch.cuda.synchronize()
    st = p.solve_device(x.data_ptr(), b.data_ptr(), raise_on_error=False)
    assert st == pps.NOT_CONVERGED, pps.status_string(st)
    d = p.stats()
    assert d["iterations"] == 2 and np.isfinite(d["err_true"]) and d["err_true"] < 1.0
    p.close()
