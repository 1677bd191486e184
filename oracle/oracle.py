"""Python access to the FP64 C oracle (``oracle/capon_oracle.c``).

TEST INFRASTRUCTURE ONLY -- the checker for the CUDA path and the CPU
baseline of the benchmark; the product never imports this module.

``build()`` compiles ``liboracle.so`` with gcc (x86 here, aarch64 on the GPU
host).  ``capon(Xd, regCoef, L, Navg, ...)`` returns a dict with
``z`` (complex128), ``zpow`` (the reference's upper-triangle power, complex128),
``P`` (true MVDR power w^H R_d w, float64), ``w`` and optionally ``R``
(loaded, normalised, full Hermitian, row-major per pixel).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "capon_oracle.c")
LIB = os.path.join(HERE, "liboracle.so")

_lib = None


def build() -> str:
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + ".tmp"
    subprocess.run(["gcc", "-O2", "-std=c11", "-shared", "-fPIC", SRC, "-o", tmp, "-lm", "-lpthread"], check=True)
    os.replace(tmp, LIB)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp, i, d = C.c_void_p, C.c_int, C.c_double
        L.oracle_capon.argtypes = [vp, i, i, i, d, i, i, i, i, i, vp, vp, vp, vp, vp, i]
        L.oracle_capon.restype = i
        L.oracle_capon_ex.argtypes = [vp, i, i, i, d, i, i, i, i, i, i, vp, vp, vp, vp, vp, i]
        L.oracle_capon_ex.restype = i
        L.oracle_capon_v.argtypes = [vp, i, i, i, d, i, i, i, i, i, i, vp, vp, vp, vp, vp, vp, i]
        L.oracle_capon_v.restype = i
        for name in ("oracle_cholesky",):
            getattr(L, name).argtypes = [vp, i, vp]
        for name in ("oracle_forward_solve", "oracle_back_solve"):
            getattr(L, name).argtypes = [vp, vp, i, vp]
        L.oracle_solve_cholesky.argtypes = [vp, vp, i, vp, vp]
        L.oracle_butler.argtypes = [i, i, vp]
        L.oracle_sm_update.argtypes = [vp, vp, i, i, vp]
        L.oracle_sm_update.restype = d
        L.oracle_sm_row.argtypes = [vp, vp, i, i, i, vp]
        L.oracle_sm_row.restype = d
        L.oracle_capon_sliding.argtypes = [vp, i, i, i, d, i, i, i, vp, vp, vp, vp, i]
        L.oracle_capon_sliding.restype = i
        L.oracle_butler_layout.argtypes = [i, i, vp, i]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data if a is not None else None


def capon(Xd, regCoef, L, Navg, Nb=0, bs_loading=False, fp32_scalars=True, want_w=True, want_R=False,
          nthreads=1, absolute=False, fb=False, V=None) -> dict:
    """absolute=True: R_d = R + regCoef*I on the normalised R instead of the
    relative loading regCoef*tr(R)/L.  fb=True: forward-backward averaged
    covariance (R + J R^T J)/2 before loading and any beamspace transform.
    V: optional Nb x L subspace matrix replacing the Butler matrix (Nb > 0)."""
    Xd = np.ascontiguousarray(Xd, dtype=np.complex64)
    Nx, Ny, M = Xd.shape
    npy = Ny - 2 * Navg
    out = dict(
        z=np.zeros((Nx, npy), np.complex128),
        zpow=np.zeros((Nx, npy), np.complex128),
        P=np.zeros((Nx, npy), np.float64),
        w=np.zeros((Nx, npy, L), np.complex128) if want_w else None,
        R=np.zeros((Nx, npy, L, L), np.complex128) if want_R else None,
    )
    mode = 2 if absolute else int(bool(bs_loading))
    Vc = None if V is None else np.ascontiguousarray(V, dtype=np.complex128)
    rc = lib().oracle_capon_v(_p(Xd), Nx, Ny, M, float(regCoef), int(L), int(Navg), int(Nb), mode,
                              int(bool(fp32_scalars)), int(bool(fb)), _p(Vc), _p(out["z"]), _p(out["zpow"]),
                              _p(out["w"]), _p(out["P"]), _p(out["R"]), int(nthreads))
    if rc != 0:
        raise ValueError(f"oracle_capon returned {rc}")
    return out


def sm_row(B, X, L, sign) -> tuple:
    """One row of rank-1 changes of an inverse, woodburyc.pyx:15-42
    (iterativeBuildUpRinv for sign=+1, iterativeBuildDownRinv for -1).
    Returns (new B, smallest denominator)."""
    B = np.array(B, dtype=np.complex128, order="C")
    X = np.ascontiguousarray(X, dtype=np.complex128)
    u = np.zeros(2 * L, np.complex128)
    den = lib().oracle_sm_row(_p(B), _p(X), X.shape[0], int(L), int(sign), _p(u))
    return B, den


def capon_sliding(Xd, d, L, Navg, segment, want_w=True, nthreads=1) -> dict:
    """Capon with the inverse tracked along range by Sherman-Morrison updates
    (getCaponAllC.pyx:240-252, woodburyc.pyx:15-107), absolute loading
    R_d = R + d I, a fresh build-up every `segment` pixels."""
    Xd = np.ascontiguousarray(Xd, dtype=np.complex64)
    Nx, Ny, M = Xd.shape
    npy = Ny - 2 * Navg
    out = dict(
        z=np.zeros((Nx, npy), np.complex128),
        P=np.zeros((Nx, npy), np.float64),
        w=np.zeros((Nx, npy, L), np.complex128) if want_w else None,
    )
    dmin = np.zeros(1, np.float64)
    rc = lib().oracle_capon_sliding(_p(Xd), Nx, Ny, M, float(d), int(L), int(Navg), int(segment), _p(out["z"]),
                                    _p(out["w"]), _p(out["P"]), _p(dmin), int(nthreads))
    if rc != 0:
        raise ValueError(f"oracle_capon_sliding returned {rc}")
    out["den_min"] = float(dmin[0])
    return out


def cholesky(A) -> np.ndarray:
    A = np.ascontiguousarray(A, dtype=np.complex128)
    n = A.shape[0]
    U = np.zeros_like(A)
    lib().oracle_cholesky(_p(A), n, _p(U))
    return U


def forward_solve(A, b) -> np.ndarray:
    A = np.ascontiguousarray(A, dtype=np.complex128)
    b = np.ascontiguousarray(b, dtype=np.complex128)
    x = np.zeros_like(b)
    lib().oracle_forward_solve(_p(A), _p(b), A.shape[0], _p(x))
    return x


def back_solve(A, b) -> np.ndarray:
    A = np.ascontiguousarray(A, dtype=np.complex128)
    b = np.ascontiguousarray(b, dtype=np.complex128)
    x = np.zeros_like(b)
    lib().oracle_back_solve(_p(A), _p(b), A.shape[0], _p(x))
    return x


def solve_cholesky(A, b) -> np.ndarray:
    A = np.ascontiguousarray(A, dtype=np.complex128)
    b = np.ascontiguousarray(b, dtype=np.complex128)
    n = A.shape[0]
    x = np.zeros_like(b)
    work = np.zeros(2 * n * n + n, np.complex128)
    lib().oracle_solve_cholesky(_p(A), _p(b), n, _p(x), _p(work))
    return x


def butler(Nb, L, symmetric=True) -> np.ndarray:
    """Nb x L Butler matrix; symmetric=True is the GPU beam layout, False the
    first Nb DFT bins (framework/linalg/beamspace.py butlerMatrix)."""
    B = np.zeros((Nb, L), np.complex128)
    lib().oracle_butler_layout(int(Nb), int(L), _p(B), int(bool(symmetric)))
    return B
