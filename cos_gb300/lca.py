"""Low-complexity adaptive (LCA) window selection on the GPU, mirroring
framework/beamformer/lca/lcac.py: ``lca(Z, wrf) -> (img, win)`` with Z the
beamformer outputs [Ny][Nx][Nw] for Nw windows and wrf the odd-sized [Yf][Xf]
averaging filter (float64)."""
from __future__ import annotations

import numpy as np

from ._lib import check, lib


def lca(Z, wrf):
    from .capon import _module_ctx
    Zc = np.ascontiguousarray(Z, dtype=np.complex64)
    w = np.ascontiguousarray(wrf, dtype=np.float64)
    if Zc.ndim != 3 or w.ndim != 2:
        raise ValueError("Z must be [Ny][Nx][Nw] and wrf 2-D")
    Ny, Nx, Nw = Zc.shape
    img = np.zeros((Ny, Nx), np.complex64)
    win = np.zeros((Ny, Nx), np.int32)
    check(lib.cos_capon_lca(_module_ctx().handle, Zc.ctypes.data, Ny, Nx, Nw, w.ctypes.data, w.shape[0], w.shape[1],
                            img.ctypes.data, win.ctypes.data, 0, None), "cos_capon_lca")
    return img, win
