"""Restatement of the reference's LCA window selection
(framework/beamformer/lca/lcac.py, general-filter and 1 x 1 branches; the same
algorithm as lcacx.pyx:175-216 with its Z[Ny][Nx][Nw] indexing).

TEST INFRASTRUCTURE ONLY -- the checker of cos_capon_lca.
"""
from __future__ import annotations

import numpy as np


def lca(Z, wrf):
    Z = np.asarray(Z)
    wrf = np.asarray(wrf, dtype=np.float64)
    Ny, Nx, Nw = Z.shape
    Yf, Xf = wrf.shape
    Ym, Xm = (Yf - 1) // 2, (Xf - 1) // 2
    if Yf == 1 and Xf == 1 and wrf[0, 0]:                      # lcac.py: argmin |Z| per pixel
        sel = np.abs(Z).argmin(2)
        return np.take_along_axis(Z, sel[..., None], 2)[..., 0], sel
    img = np.zeros((Ny, Nx), Z.dtype)
    win = np.zeros((Ny, Nx), int)
    p = np.abs(Z) ** 2                                          # img_abs, [Ny][Nx][Nw]
    sums = np.zeros((Ny, Nx, Nw))
    for yy in range(Yf):
        for xx in range(Xf):
            sums[Ym:Ny - Ym, Xm:Nx - Xm] += wrf[yy, xx] * p[yy:Ny - Yf + 1 + yy, xx:Nx - Xf + 1 + xx]
    sel = sums.argmin(2)                                        # first minimum, as `<` in the loop
    inner = (slice(Ym, Ny - Ym), slice(Xm, Nx - Xm))
    win[inner] = sel[inner]
    img[inner] = np.take_along_axis(Z, sel[..., None], 2)[..., 0][inner]
    return img, win, sums
