"""Training pipeline of the learned preconditioner.

(f, u) pairs: f is a seeded k^-2 Gaussian random field or a sum of 1-8 Gaussian
blobs, u the solution of -lap u = f with Dirichlet zero boundaries.  Two operators:
the solver's own grid (u from the plain FP64 GPU solver to ||r||/||b|| <= 1e-12), or,
for the coarsest level of the multigrid cycle after k coarsenings of an even grid,
the level operator whose upper wall sits 2^-k spacings above the last unknown (u
from an exact tensor-product eigen-solve).  The network learns the map from b = -f
(scaled to unit RMS) to u / (rms(b) * S), S a dataset-wide scale, so that gain = S
turns its output back into a solution: u ~ S * rms(b) * N(b / rms(b)).  Training
and inference run on the library's own kernels (pps_unet_*).
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


def level_operator_1d(n: int, gap: float) -> np.ndarray:
    """Second difference at unit spacing on n unknowns, the lower wall one spacing
    below the first unknown and the upper wall `gap` spacings above the last (the
    three-point formula for unequal spacings there); gap = 1 is the uniform grid."""
    t = np.zeros((n, n))
    for i in range(n):
        t[i, i] = -2.0
        if i > 0:
            t[i, i - 1] = 1.0
        if i + 1 < n:
            t[i, i + 1] = 1.0
    t[n - 1, n - 2] = 2.0 / (1.0 + gap) if n > 1 else 0.0
    t[n - 1, n - 1] = -2.0 / gap
    return t


def level_solve(b, h: float, gap: float):
    """u with A u = b on an n^3 cube, A the sum over axes of level_operator_1d / h^2;
    b: (..., n, n, n) float64 torch tensor.  Exact: the 1-D operator is diagonalisable
    (tridiagonal with positive off-diagonal products), so A is in the tensor basis."""
    import torch
    n = b.shape[-1]
    w, v = np.linalg.eig(level_operator_1d(n, gap))
    w, v = w.real, v.real
    vi = np.linalg.inv(v)
    V = torch.from_numpy(v).to(b)
    Vi = torch.from_numpy(vi).to(b)
    lam = torch.from_numpy(w).to(b) / (h * h)
    bt = torch.einsum("ai,bj,ck,...ijk->...abc", Vi, Vi, Vi, b)
    den = lam[:, None, None] + lam[None, :, None] + lam[None, None, :]
    return torch.einsum("ai,bj,ck,...ijk->...abc", V, V, V, bt / den)


def make_dataset(m: int, seeds, device: int = 0, tol: float = 1e-12, coarsen: int | None = None):
    """List of (b, u) dense float32 CUDA tensors of the m^3 unknowns; even seeds are
    random fields, odd seeds blobs.  With `coarsen` = k, u solves the coarse-level
    operator of k coarsenings (upper wall 2^-k spacings above the last unknown)."""
    import torch
    if coarsen is not None:
        out = []
        inner = (slice(2, m + 2),) * 3
        h = 1.0 / (m + 1)
        for sd in seeds:
            b = torch.from_numpy(np.ascontiguousarray(rhs(m, int(sd), "field" if sd % 2 == 0 else "blobs")[inner]))
            bd = b.cuda(device)
            u = level_solve(bd, h, 2.0 ** (-coarsen))
            out.append((bd.float().contiguous(), u.float().contiguous()))
        return out
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


def make_dataset_batch(m: int, seed: int, count: int, coarsen: int, device=0, chunk: int = 2048):
    """`count` (b, u) pairs for the coarse level of `coarsen` coarsenings, generated
    in batches from one seeded torch generator on `device` (a CUDA ordinal, or a torch
    device): the first half k^-2 random fields (the distribution of random_field), the
    second half sums of 1-8 Gaussian blobs (that of blobs); u from the exact level
    solve.  Returns a list of dense float32 tensor pairs like make_dataset."""
    import torch
    dev = torch.device("cuda", device) if isinstance(device, int) else torch.device(device)
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed))
    h = 1.0 / (m + 1)
    gap = 2.0 ** (-coarsen)
    kz = torch.fft.fftfreq(m, d=1.0 / m, dtype=torch.float64, device=dev)
    kx = torch.fft.rfftfreq(m, d=1.0 / m, dtype=torch.float64, device=dev)
    k2 = kz[:, None, None] ** 2 + kz[None, :, None] ** 2 + kx[None, None, :] ** 2
    amp = torch.where(k2 > 0, k2 ** (-2.0 / 4.0), torch.zeros_like(k2))
    c = torch.arange(1, m + 1, dtype=torch.float64, device=dev) * h
    out = []
    n_field = count // 2
    done = 0
    while done < count:
        nb = min(chunk, count - done)
        nf = max(0, min(nb, n_field - done))   # random fields in this batch
        parts = []
        if nf > 0:
            noise = torch.randn((nf, m, m, m), generator=gen, dtype=torch.float64, device=dev)
            f = torch.fft.irfftn(torch.fft.rfftn(noise, dim=(1, 2, 3)) * amp, s=(m, m, m), dim=(1, 2, 3))
            f = f / torch.sqrt(torch.mean(f * f, dim=(1, 2, 3), keepdim=True))
            parts.append(-f)
        ng = nb - nf
        if ng > 0:
            nblob = torch.randint(1, 9, (ng, 1), generator=gen, device=dev)
            active = (torch.arange(8, device=dev)[None, :] < nblob).to(torch.float64)
            ctr = 0.2 + 0.6 * torch.rand((ng, 8, 3), generator=gen, dtype=torch.float64, device=dev)
            w = 0.02 + 0.08 * torch.rand((ng, 8), generator=gen, dtype=torch.float64, device=dev)
            a = torch.randn((ng, 8), generator=gen, dtype=torch.float64, device=dev) * active
            g = torch.exp(-((c[None, None, None, :] - ctr[..., None]) ** 2) / (2 * w[..., None, None] ** 2))
            f = torch.einsum("bk,bkz,bky,bkx->bzyx", a, g[:, :, 2], g[:, :, 1], g[:, :, 0])
            parts.append(-f)
        b = torch.cat(parts, 0)
        u = level_solve(b, h, gap)
        for i in range(nb):
            out.append((b[i].float().contiguous(), u[i].float().contiguous()))
        done += nb
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
    torch.cuda.synchronize()   # the network's stream does not wait for torch's
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
    torch.cuda.synchronize()   # the network's stream does not wait for torch's
    for b, u in data:
        out = torch.empty_like(b)
        net.forward(tuple(b.shape), b.data_ptr(), out.data_ptr(), normalize=True)
        torch.cuda.synchronize()
        pred = out * scale
        errs.append(float(torch.linalg.norm(pred - u) / torch.linalg.norm(u)))
    return errs
