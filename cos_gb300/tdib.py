"""Time-domain steering (TDIB) on the GPU: the step that produces the Capon
input cube, mirroring framework/beamformer/delay/tdibC.pyx:9-67.

* ``tdib(mfdata, mtaxe, x_r, D, c, fc, xarr, yarr) -> image`` -- the
  reference's signature and result: the delay-and-sum image [n_y][n_x]
  (the mean over hydrophones of the steered samples).
* ``steer(...) -> Xd`` -- the steered per-channel cube [n_x][n_y][n_hydros]
  (complex64), the input layout of ``getCaponGPU`` / ``cos_capon_run``.

mtaxe must be uniform (t0 + k dt); samples outside it are NaN, as the
reference's interp1d(bounds_error=False) gives.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from ._lib import check, lib


def _axis(mtaxe):
    t = np.asarray(mtaxe, dtype=np.float64)
    if t.ndim != 1 or t.size < 2:
        raise ValueError("mtaxe must be a 1-D time axis of at least 2 samples")
    dt = (t[-1] - t[0]) / (t.size - 1)
    if not dt > 0 or np.abs(t - (t[0] + dt * np.arange(t.size))).max() > 1e-9 * abs(t[-1] - t[0]):
        raise ValueError("mtaxe must be uniform and increasing")
    return float(t[0]), float(dt)


def _run(mfdata, mtaxe, x_r, D, c, fc, xarr, yarr, want_xd, want_image):
    from .capon import _module_ctx
    mf = np.ascontiguousarray(mfdata, dtype=np.complex64)
    if mf.ndim == 3:   # several banks: the first, as tdibC.pyx:12-16
        mf = np.ascontiguousarray(mf[:, :, 1] if mf.shape[2] > 1 else mf[:, :, 0])
    n_h, n_s = mf.shape
    t0, dt = _axis(mtaxe)
    xr = np.ascontiguousarray(x_r, dtype=np.float64).reshape(-1)
    dd = np.ascontiguousarray(D, dtype=np.float64).reshape(-1)
    xa = np.ascontiguousarray(xarr, dtype=np.float64)
    ya = np.ascontiguousarray(yarr, dtype=np.float64)
    if xa.shape != ya.shape or xa.ndim != 2 or xr.size != n_h or dd.size != n_h:
        raise ValueError("xarr/yarr must be [n_x][n_y]; x_r and D one value per hydrophone")
    n_x, n_y = xa.shape
    Xd = np.zeros((n_x, n_y, n_h), np.complex64) if want_xd else None
    img = np.zeros((n_y, n_x), np.complex64) if want_image else None
    ptr = lambda a: a.ctypes.data if a is not None else None   # noqa: E731
    check(lib.cos_capon_tdib(_module_ctx().handle, ptr(mf), n_h, n_s, t0, dt, ptr(xr), ptr(dd), float(c),
                             float(fc), ptr(xa), ptr(ya), n_x, n_y, ptr(Xd), ptr(img), 0, None), "cos_capon_tdib")
    return Xd, img


def tdib(mfdata, mtaxe, x_r, D, c, fc, xarr, yarr):
    """Delay-and-sum image [n_y][n_x] (complex64), tdibC.pyx's result."""
    return _run(mfdata, mtaxe, x_r, D, c, fc, xarr, yarr, False, True)[1]


def steer(mfdata, mtaxe, x_r, D, c, fc, xarr, yarr):
    """Steered cube Xd [n_x][n_y][n_hydros] (complex64)."""
    return _run(mfdata, mtaxe, x_r, D, c, fc, xarr, yarr, True, False)[0]
