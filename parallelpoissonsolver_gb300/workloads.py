"""Seeded synthetic right-hand sides of the benchmark configurations.

The reference publishes no dataset; these stand in for its benchmark inputs with
the shapes, sizes and value distributions the configurations name.  All fields
are guard-padded float64 arrays (n+2)^3 with the unknowns in [2, n) of an
npglobal = m+2 grid (m unknowns per axis, h = 1/(m+1), Dirichlet 0), and hold
b = -f for -lap u = f, because the solver's operator is the positive-sign
Laplacian (matrixFreeOperatorA.hpp:33-38).

* random_field(m, seed, slope): white noise N(0,1) filtered in Fourier space to a
  power spectrum P(k) ~ k^slope (amplitude |k|^(slope/2) on integer wavevectors,
  k = 0 removed), normalised to unit RMS.  The 512^3 benchmark field uses slope -2,
  the 1024^3 charges workload's background slope -3 at RMS 0.1.
* blobs(m, seed): a sum of 1-8 Gaussian blobs, centres U[0.2,0.8]^3, widths
  U[0.02,0.1], amplitudes N(0,1) (the batched workload).
* charges(m, seed, count): point-like Gaussian charges of width 2h, amplitudes +-1,
  centres uniform (the 1024^3 workload).
"""
from __future__ import annotations

import numpy as np


def _interior(m: int, values: np.ndarray) -> np.ndarray:
    b = np.zeros((m + 4,) * 3, np.float64)
    b[2:m + 2, 2:m + 2, 2:m + 2] = values
    return b


def _random_field_tensor(m: int, seed: int, slope: float, dev):
    """The random field of random_field_values as a float64 torch tensor on `dev`."""
    import torch
    rng = np.random.default_rng(seed)
    t = torch.from_numpy(rng.standard_normal((m, m, m))).to(dev)
    F = torch.fft.rfftn(t)
    del t
    kz = torch.fft.fftfreq(m, d=1.0 / m, dtype=torch.float64, device=dev)
    kx = torch.fft.rfftfreq(m, d=1.0 / m, dtype=torch.float64, device=dev)
    k2 = kz[:, None, None] ** 2 + kz[None, :, None] ** 2 + kx[None, None, :] ** 2
    amp = torch.where(k2 > 0, k2 ** (slope / 4.0), torch.zeros_like(k2))
    F = F * amp
    del amp, k2
    out = torch.fft.irfftn(F, s=(m, m, m))
    del F
    return out / torch.sqrt(torch.mean(out * out))


def random_field_values(m: int, seed: int, slope: float = -2.0, device=None) -> np.ndarray:
    """m^3 unit-RMS Gaussian random field with P(k) ~ k^slope (float64, z,y,x order)."""
    try:
        import torch
        dev = device if device is not None else ("cuda" if torch.cuda.is_available() else "cpu")
        return _random_field_tensor(m, seed, slope, dev).cpu().numpy()
    except ImportError:
        rng = np.random.default_rng(seed)
        noise = rng.standard_normal((m, m, m))
        F = np.fft.rfftn(noise)
        kz = np.fft.fftfreq(m, d=1.0 / m)
        kx = np.fft.rfftfreq(m, d=1.0 / m)
        k2 = kz[:, None, None] ** 2 + kz[None, :, None] ** 2 + kx[None, None, :] ** 2
        with np.errstate(divide="ignore"):
            amp = np.where(k2 > 0, k2 ** (slope / 4.0), 0.0)
        out = np.fft.irfftn(F * amp, s=(m, m, m))
        return out / np.sqrt(np.mean(out * out))


def random_field(m: int, seed: int = 2, slope: float = -2.0, rms: float = 1.0, device=None) -> np.ndarray:
    """Guard-padded b = -f for f a random field (the 512^3 benchmark: seed 2, slope -2)."""
    return _interior(m, -rms * random_field_values(m, seed, slope, device))


def _coords(m: int):
    h = 1.0 / (m + 1)
    c = np.arange(1, m + 1) * h   # interior nodes 2..m+1 sit at (i-1)*h, i.e. h..m*h
    return c


def blobs(m: int, seed: int) -> np.ndarray:
    """Guard-padded b = -f for a seeded sum of 1-8 Gaussian blobs (the batched workload)."""
    rng = np.random.default_rng(seed)
    nb = int(rng.integers(1, 9))
    c = _coords(m)
    f = np.zeros((m, m, m))
    for _ in range(nb):
        cx, cy, cz = rng.uniform(0.2, 0.8, 3)
        w = rng.uniform(0.02, 0.1)
        a = rng.standard_normal()
        gx = np.exp(-((c - cx) ** 2) / (2 * w * w))
        gy = np.exp(-((c - cy) ** 2) / (2 * w * w))
        gz = np.exp(-((c - cz) ** 2) / (2 * w * w))
        f += a * gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
    return _interior(m, -f)


def charges(m: int, seed: int = 5, count: int = 64, background_rms: float = 0.1) -> np.ndarray:
    """Guard-padded b = -f: `count` Gaussian charges of width 2h, amplitude +-1, plus a
    k^-3 random-field background at the given RMS (the 1024^3 workload)."""
    rng = np.random.default_rng(seed)
    h = 1.0 / (m + 1)
    c = _coords(m)
    f = background_rms * random_field_values(m, seed + 1000, -3.0)
    w = 2 * h
    for _ in range(count):
        cx, cy, cz = rng.uniform(0.0, 1.0, 3)
        a = rng.choice([-1.0, 1.0])
        gx = np.exp(-((c - cx) ** 2) / (2 * w * w))
        gy = np.exp(-((c - cy) ** 2) / (2 * w * w))
        gz = np.exp(-((c - cz) ** 2) / (2 * w * w))
        f += a * gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
    return _interior(m, -f)


def charges_device(m: int, seed: int = 5, count: int = 64, background_rms: float = 0.1, device="cuda"):
    """charges() built on the GPU as a guard-padded float64 torch tensor (the 1024^3
    case: 8.6 GB per field)."""
    import torch
    rng = np.random.default_rng(seed)
    h = 1.0 / (m + 1)
    c = torch.arange(1, m + 1, dtype=torch.float64, device=device) * h
    f = background_rms * _random_field_tensor(m, seed + 1000, -3.0, device)
    w = 2 * h
    for _ in range(count):
        cx, cy, cz = rng.uniform(0.0, 1.0, 3)
        a = rng.choice([-1.0, 1.0])
        gx = torch.exp(-((c - cx) ** 2) / (2 * w * w))
        gy = torch.exp(-((c - cy) ** 2) / (2 * w * w))
        gz = torch.exp(-((c - cz) ** 2) / (2 * w * w))
        f.add_(a * gz[:, None, None] * gy[None, :, None] * gx[None, None, :])
    b = torch.zeros((m + 4,) * 3, dtype=torch.float64, device=device)
    b[2:m + 2, 2:m + 2, 2:m + 2] = -f
    return b


def batch_edges(count: int = 256, seed: int = 3):
    """Grid edges of the batched configuration: uniform on {32,48,64,96,128}."""
    rng = np.random.default_rng(seed)
    return [int(v) for v in rng.choice([32, 48, 64, 96, 128], count)]
