"""Seeded synthetic data cubes for the Capon path.

The reference's own data (sonar / ultrasound .mat datasets loaded through
framework/fileLUT.py) is not available, so cubes are generated:

* noise: circular complex Gaussian, E|n|^2 = sigma^2;
* each scatterer at (y0, b0) with amplitude A adds
  A * exp(-(y-y0)^2 / (2*4^2)) * exp(j*pi*(b-b0)*m*2/M) to cube[y, b, m]
  (a plane-wave phase ramp across channels that is flat on its own beam and
  advances by one DFT bin of the M-element aperture per beam of offset);
* positions are drawn by the seed, y0 in [12, Ny-12], b0 in [0, Nx).

Cubes are generated [Ny, Nx, M] and returned as the entry points take them,
Xd[Nx][Ny][M] (getCaponC.pyx:74-76) -- C-contiguous complex64.
"""
from __future__ import annotations

import numpy as np

SIGMA_Y = 4.0


def cube(Ny: int, Nx: int, M: int, amplitudes, seed: int, sigma: float = 1.0, coherent_pair: bool = False,
         dtype=np.complex64) -> np.ndarray:
    rng = np.random.default_rng(seed)
    n = (rng.standard_normal((Ny, Nx, M), dtype=np.float32) +
         1j * rng.standard_normal((Ny, Nx, M), dtype=np.float32)) * np.float32(sigma / np.sqrt(2.0))
    c = n.astype(np.complex64)
    y = np.arange(Ny, dtype=np.float64)[:, None, None]
    b = np.arange(Nx, dtype=np.float64)[None, :, None]
    m = np.arange(M, dtype=np.float64)[None, None, :]
    lo, hi = 3 * SIGMA_Y, Ny - 3 * SIGMA_Y
    if coherent_pair:
        # two fully coherent scatterers (same phase), one beam apart, same range
        y0 = rng.uniform(lo, hi)
        b0 = int(rng.integers(0, max(1, Nx - 1)))
        pos = [(y0, b0), (y0, b0 + 1)]
    else:
        pos = [(rng.uniform(lo, hi), int(rng.integers(0, Nx))) for _ in amplitudes]
    for A, (y0, b0) in zip(amplitudes, pos):
        env = np.exp(-((y - y0) ** 2) / (2 * SIGMA_Y ** 2))
        rows = np.nonzero(env[:, 0, 0] > 1e-12)[0]
        r0, r1 = int(rows.min()), int(rows.max()) + 1
        ph = np.exp(1j * np.pi * (b - b0) * m * (2.0 / M))
        c[r0:r1] += (A * env[r0:r1] * ph).astype(np.complex64)
    return np.ascontiguousarray(c.transpose(1, 0, 2))


def config0(seed: int = 0) -> dict:
    """Plain element-space MVDR, small: [Ny=512, Nx=128, M=32], A = 10, 5, 3;
    L=16, K=1, loading 0.01."""
    return dict(x=cube(512, 128, 32, [10.0, 5.0, 3.0], seed), L=16, K=1, d=0.01, Nb=0)


def config1(seed: int = 1, Ny: int = 2048, Nx: int = 256) -> dict:
    """Throughput: [Ny=2048, Nx=256, M=64], 8 scatterers at 20 dB per element;
    L=32, K=2, loading 0.01."""
    return dict(x=cube(Ny, Nx, 64, [10.0] * 8, seed), L=32, K=2, d=0.01, Nb=0)


def config2(seed: int = 2, Ny: int = 1024, Nx: int = 256) -> list:
    """Uneven frames in one launch: (M, L, Nb) = (32,16,0), (64,32,0),
    (96,48,3), (128,64,5); Ny=1024, Nx=256, K=1, loading 0.01."""
    out = []
    for i, (M, L, Nb) in enumerate([(32, 16, 0), (64, 32, 0), (96, 48, 3), (128, 64, 5)]):
        out.append(dict(x=cube(Ny, Nx, M, [10.0, 5.0, 3.0], seed * 10 + i), L=L, K=1, d=0.01, Nb=Nb))
    return out


def config3(seed: int = 3, Ny: int = 2048, Nx: int = 256) -> dict:
    """Precision stress: [2048, 256, 128], two fully coherent scatterers one
    beam apart at 40 dB; L=64, K=4, loading 1e-3."""
    return dict(x=cube(Ny, Nx, 128, [100.0, 100.0], seed, coherent_pair=True), L=64, K=4, d=1e-3, Nb=0)
