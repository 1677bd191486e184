"""FP64 restatement of the reference's time-domain steering
(framework/beamformer/delay/tdibC.pyx:9-67).

TEST INFRASTRUCTURE ONLY -- the checker of cos_capon_tdib; the product never
imports this module.

steer() returns the per-hydrophone terms the reference sums (the interpolated,
carrier-mixed samples, tdibC.pyx:40-58) as a cube [n_x][n_y][n_hydros];
tdib() returns the reference's result, image.T / n_hydros (:61-67).  Linear
interpolation with NaN outside the time axis is np.interp with left/right NaN,
the semantics of scipy's interp1d(kind='linear', bounds_error=False).
"""
from __future__ import annotations

import numpy as np


def steer(mfdata, mtaxe, x_r, D, c, fc, xarr, yarr):
    mf = np.asarray(mfdata)
    n_h = mf.shape[0]
    xarr = np.asarray(xarr, dtype=np.float64)
    yarr = np.asarray(yarr, dtype=np.float64)
    n_x, n_y = xarr.shape
    t = np.asarray(mtaxe, dtype=np.float64)
    xx = np.mean(x_r) / 2          # tdibC.pyx:29-30
    zz = np.mean(D) / 2
    out = np.zeros((n_x, n_y, n_h), np.complex128)
    for nx in range(n_x):
        r_t = np.sqrt((xx + xarr[nx]) ** 2 + yarr[nx] ** 2 + zz ** 2)                     # :36
        for n in range(n_h):
            r_r = np.sqrt((xx + xarr[nx] - x_r[n]) ** 2 + yarr[nx] ** 2 + (zz - D[n]) ** 2)   # :42
            tipos = (r_t + r_r) * (1.0 / c)                                                 # :25, :45
            re = np.interp(tipos, t, mf[n].real.astype(np.float64), left=np.nan, right=np.nan)
            im = np.interp(tipos, t, mf[n].imag.astype(np.float64), left=np.nan, right=np.nan)
            out[nx, :, n] = (re + 1j * im) * np.exp(2j * np.pi * fc * tipos)                 # :58
    return out


def tdib(mfdata, mtaxe, x_r, D, c, fc, xarr, yarr):
    return steer(mfdata, mtaxe, x_r, D, c, fc, xarr, yarr).sum(axis=2).T / np.asarray(mfdata).shape[0]


def scenario(seed=0, n_h=16, n_s=2048, n_x=8, n_y=128, fs=50e3, fc=100e3, c=1480.0):
    """A seeded SAS-like geometry: a line array, pixels at 20-60 m slant range,
    matched-filtered data with point echoes (for the tests and the bench)."""
    rng = np.random.default_rng(seed)
    x_r = np.linspace(-0.5, 0.5, n_h) * 0.04 * n_h
    D = 0.02 * rng.standard_normal(n_h)
    t = 2 * 15.0 / c + np.arange(n_s) / fs
    xarr = np.repeat(np.linspace(-2.0, 2.0, n_x)[:, None], n_y, axis=1)
    # slant ranges whose two-way delays (with the array and beam offsets) stay
    # inside the recorded time axis
    y0, y1 = 1.02 * t[0] * c / 2 + 1.0, 0.97 * t[-1] * c / 2
    yarr = np.repeat(np.linspace(y0, y1, n_y)[None, :], n_x, axis=0)
    mf = (rng.standard_normal((n_h, n_s)) + 1j * rng.standard_normal((n_h, n_s))) * 0.1
    for _ in range(5):   # echoes: Gaussian pulses at random delays
        k0 = rng.uniform(100, n_s - 100)
        k = np.arange(n_s)
        mf += 3.0 * np.exp(-0.5 * ((k - k0) / 3.0) ** 2) * np.exp(1j * rng.uniform(0, 2 * np.pi, (n_h, 1)))
    return dict(mfdata=mf.astype(np.complex64), mtaxe=t, x_r=x_r, D=D, c=c, fc=fc, xarr=xarr, yarr=yarr)
