"""Training pipeline of the learned preconditioner.

(f, u) pairs: f is a seeded k^-2 Gaussian random field or a sum of 1-8 Gaussian
blobs, u the solution of -lap u = f with Dirichlet zero boundaries, solved by the
plain FP64 GPU solver to ||r||/||b|| <= 1e-12.  The network learns the map from
b = -f (scaled to unit RMS) to u / (rms(b) * S), S a dataset-wide scale, so that
gain = S turns its output back into a solution: u ~ S * rms(b) * N(b / rms(b)).
Training and inference run on the library's own kernels (pps_unet_*).
"""
from __future__ import annotations

import time

import numpy as np

import parallelpoissonsolver_gb300 as pps
from parallelpoissonsolver_gb300 import workloads


def rhs(m: int, seed: int, kind: str) -> np.ndarray:
    if kind == "field":
        return workloads.random_field(m, seed=seed, slope=-2.0)
    return workloads.blobs(m, seed)


def make_dataset(m: int, seeds, device: int = 0, tol: float = 1e-12):
    """List of (b, u) dense float32 CUDA tensors of the m^3 unknowns; even seeds are
    random fields, odd seeds blobs."""
    import torch
    grid = pps.BlockGrid.cube(m)
    solver = pps.BiCGSTAB(grid, pps.ChebyshevIteration(11), tolerance=tol, max_iteration=20000, form="fp64",
                          device=device)
    out = []
    inner = (slice(2, m + 2),) * 3
    for sd in seeds:
        b = rhs(m, int(sd), "field" if sd % 2 == 0 else "blobs")
        bd = torch.from_numpy(b).cuda(device)
        xd = torch.zeros_like(bd)
        torch.cuda.synchronize()
        st = solver.solve_device(xd.data_ptr(), bd.data_ptr())
        if st != pps.OK:
            raise RuntimeError(f"training solve {sd}: {pps.status_string(st)}")
        out.append((bd[inner].float().contiguous(), xd[inner].float().contiguous()))
    solver.close()
    return out


def fit_scale(data) -> float:
    import torch
    r = [float(torch.sqrt(torch.mean(u * u)) / torch.sqrt(torch.mean(b * b))) for b, u in data]
    return float(np.median(r))


def train(net: "pps.UNet", data, scale: float, steps: int, lr: float = 2e-3, seed: int = 0, log_every: int = 0):
    """Adam steps of batch size 1 over shuffled samples; returns the loss history."""
    import torch
    rng = np.random.default_rng(seed)
    prepared = []
    for b, u in data:
        rb = torch.sqrt(torch.mean(b * b))
        prepared.append(((b / rb).contiguous(), (u / (rb * scale)).contiguous()))
    shape = tuple(data[0][0].shape)
    losses = []
    t0 = time.perf_counter()
    for k in range(steps):
        bi, ti = prepared[int(rng.integers(len(prepared)))]
        warm = min(1.0, (k + 1) / max(1, steps // 20))     # linear warm-up over 5% of the steps
        lr_k = lr * warm * (0.1 ** (k / max(steps, 1)))     # then exponential decay to lr/10
        losses.append(net.train_step(shape, bi.data_ptr(), ti.data_ptr(), lr_k))
        if log_every and (k + 1) % log_every == 0:
            print(f"step {k + 1}: loss {np.mean(losses[-log_every:]):.4e} ({time.perf_counter() - t0:.1f} s)",
                  flush=True)
    return losses


def evaluate(net: "pps.UNet", data, scale: float):
    """Relative L2 error of scale * rms(b) * N(b/rms(b)) against u for each sample."""
    import torch
    errs = []
    for b, u in data:
        out = torch.empty_like(b)
        net.forward(tuple(b.shape), b.data_ptr(), out.data_ptr(), normalize=True)
        torch.cuda.synchronize()
        pred = out * scale
        errs.append(float(torch.linalg.norm(pred - u) / torch.linalg.norm(u)))
    return errs
