"""Host-side mirror of the reference's Capon interface, on the C ABI.

Same names, argument meaning and error behaviour as the reference:

* ``Capon().getCapon(z, w, R, x, d, L, Yavg, M, Nx, Nz, Nb) -> int``
  -- ``ICapon::getCapon`` (RealTimeCapon/ICapon.h:20-33) as bound by
  RealTimeCapon/Capon.pxd:8-24; returns the CUDA error number, 0 on success.
* ``BuildR().getR(...)`` and ``Solver().solve(...)`` -- the stage interfaces
  (IBuildR.h:85-98, ISolver.h:119-128).
* ``getCaponCUDAPy(Xd, d, L, Navg, V, doFBAvg, verbose) -> [z, R, w, e]``
  -- framework/beamformer/capon/getCaponCUDA.pyx:10-81 (Nb = V.shape[0] when V
  is 2-D; doFBAvg and verbose are accepted and ignored, as there).
* ``getCaponGPU(Xd, regCoef, L, Navg, V=None, ...) -> [z, P, w]`` -- the
  argument order of getCaponC.getCaponCPy (getCaponC.pyx:61-94), returning the
  real MVDR power P = 1/Re(a^H R_d^-1 a) where the CPU path returns its
  upper-triangle sum zPow (getCaponC.pyx:285-289).
* ``capon_frames(frames, ...)`` -- the device-pointer, multi-frame call on
  torch CUDA tensors (``cos_capon_run``).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import CaponError, Frame, Opts, check, lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def opts(form: int = _lib.FORM_FUSED, loading: int = _lib.LOAD_ELEMENT, r_layout: int = _lib.R_REFERENCE,
         refine: int = 0, fb: int = 0, segment: int = 0) -> Opts:
    return Opts(form, loading, r_layout, refine, fb, segment)


class Context:
    """Owns a ``cos_capon_ctx`` (device buffer cache, stream, status word)."""

    def __init__(self):
        h = C.c_void_p()
        check(lib.cos_capon_create(C.byref(h)), "cos_capon_create")
        self.handle = h

    def close(self):
        if self.handle:
            lib.cos_capon_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def device_status(self) -> int:
        return lib.cos_capon_device_status(self.handle)


class Capon(Context):
    """Drop-in for the reference's ``Capon`` class (RealTimeCapon/Capon.pxd)."""

    def getCapon(self, z, w, R, x, d, L, Yavg, M, Nx, Nz, Nb) -> int:
        """Host arrays (complex64, C-contiguous): z [Nx][Nz-2Yavg], w [..][L],
        R [..][L][L] or None, x [Nx][Nz][M].  Returns the status code."""
        return lib.cos_capon_get_capon(self.handle, _ptr(z), _ptr(w), _ptr(R) if R is not None else None,
                                       _ptr(x), float(d), int(L), int(Yavg), int(M), int(Nx), int(Nz), int(Nb))

    def getCaponEx(self, z, P, w, R, x, d, L, Yavg, M, Nx, Nz, Nb, o: Optional[Opts] = None) -> int:
        return lib.cos_capon_get_capon_ex(
            self.handle, _ptr(z), _ptr(P) if P is not None else None, _ptr(w) if w is not None else None,
            _ptr(R) if R is not None else None, _ptr(x), float(d), int(L), int(Yavg), int(M), int(Nx),
            int(Nz), int(Nb), C.byref(o) if o is not None else None)


class BuildR(Context):
    """Drop-in for ``IBuildR::getR`` (IBuildR.h:85-98): covariance per pixel,
    column-major, loaded, not normalised."""

    def getR(self, R, x, d, L, Yavg, M, Nx, Nz, Nb, R_on_gpu=False, x_on_gpu=False) -> int:
        rp = R if R_on_gpu else _ptr(R)
        xp = x if x_on_gpu else _ptr(x)
        return lib.cos_capon_build_r(self.handle, rp, xp, float(d), int(L), int(Yavg), int(M), int(Nx),
                                     int(Nz), int(Nb), int(bool(R_on_gpu)), int(bool(x_on_gpu)))


class Solver(Context):
    """Drop-in for ``ISolver::solve`` (ISolver.h:119-128): batched A x = b,
    A column-major per system, pivoted LU."""

    def solve(self, x, A, b, N, batch, x_on_gpu=False, A_on_gpu=False, b_on_gpu=False) -> int:
        return lib.cos_capon_solve(self.handle, x if x_on_gpu else _ptr(x), A if A_on_gpu else _ptr(A),
                                   b if b_on_gpu else _ptr(b), int(N), int(batch), int(bool(x_on_gpu)),
                                   int(bool(A_on_gpu)), int(bool(b_on_gpu)))


def butler_matrix(Nb: int, L: int) -> np.ndarray:
    """Butler matrix (Nb x L complex64) computed on the GPU
    (capon_kernel.cu:47-77 beam layout)."""
    ctx = _module_ctx()
    B = np.zeros((Nb, L), np.complex64)
    check(lib.cos_capon_butler(ctx.handle, _ptr(B), int(Nb), int(L), 0), "cos_capon_butler")
    return B


_CTX: Optional[Capon] = None


def _module_ctx() -> Capon:
    # one module-level object, as getCaponCUDA.pyx:7 keeps one Capon
    global _CTX
    if _CTX is None:
        _CTX = Capon()
    return _CTX


def getCaponCUDAPy(Xd, d, L, Navg, V, doFBAvg=False, verbose=False, want_R: bool = True):
    """Mirror of getCaponCUDA.getCaponCUDAPy: returns [z, R, w, e] (complex64;
    R per pixel as the reference GPU writes it, or None with want_R=False)."""
    Xd = np.ascontiguousarray(Xd, dtype=np.complex64)
    Nx, Ny, M = Xd.shape
    L, Navg = int(L), int(Navg)
    Nb = int(V.shape[0]) if (V is not None and np.ndim(V) == 2) else 0
    z = np.zeros((Nx, Ny - 2 * Navg), np.complex64)
    w = np.zeros((Nx, Ny - 2 * Navg, L), np.complex64)
    R = np.zeros((Nx, Ny - 2 * Navg, L, L), np.complex64) if want_R else None
    e = _module_ctx().getCapon(z, w, R, Xd, float(d), L, Navg, M, Nx, Ny, Nb)
    return [z, R, w, e]


def getCaponGPU(Xd, regCoef, L, Navg, V=None, doFBAvg=False, verbose=False, *, form=_lib.FORM_FUSED,
                loading=_lib.LOAD_ELEMENT, want_w: bool = True, subspace=None, segment: int = 0,
                refine: int = _lib.REFINE_NONE):
    """getCaponCPy argument order on the GPU path: returns [z, P, w]
    (complex64 z, float32 P, complex64 w or None).  doFBAvg applies
    forward-backward averaging (the reference CPU path accepts the flag and
    ignores it, getCaponC.pyx:106; its definition is getCaponAllC.pyx:346-347).
    V, as in the reference GPU path, gives only the beam count Nb = V.shape[0]
    (the Butler matrix is used); `subspace` (complex [Nb][L]) is a caller-given
    subspace matrix with getCaponAllC.pyx:226-231, 365-370 semantics.
    `segment` sets the build-up interval of FORM_SLIDING_INVERSE.  `refine`
    (REFINE_ALL, REFINE_ADAPTIVE) adds the FP64-residual refinement step.
    Raises CaponError on a nonzero status."""
    Xd = np.ascontiguousarray(Xd, dtype=np.complex64)
    Nx, Ny, M = Xd.shape
    L, Navg = int(L), int(Navg)
    Nb = int(V.shape[0]) if (V is not None and np.ndim(V) == 2) else 0
    z = np.zeros((Nx, Ny - 2 * Navg), np.complex64)
    P = np.zeros((Nx, Ny - 2 * Navg), np.float32)
    w = np.zeros((Nx, Ny - 2 * Navg, L), np.complex64) if want_w else None
    if subspace is not None:
        Vs = np.ascontiguousarray(subspace, dtype=np.complex64)
        if Vs.ndim != 2 or Vs.shape[1] != L:
            raise ValueError("subspace must be [Nb][L]")
        o = opts(form=form, loading=loading, fb=int(bool(doFBAvg)), segment=segment, refine=refine)
        check(lib.cos_capon_get_capon_subspace(_module_ctx().handle, _ptr(z), _ptr(P),
                                               _ptr(w) if w is not None else None, _ptr(Xd), _ptr(Vs),
                                               float(regCoef), L, Navg, M, Nx, Ny, int(Vs.shape[0]), C.byref(o)),
              "cos_capon_get_capon_subspace")
        return [z, P, w]
    check(_module_ctx().getCaponEx(z, P, w, None, Xd, float(regCoef), L, Navg, M, Nx, Ny, Nb,
                                   opts(form=form, loading=loading, fb=int(bool(doFBAvg)), segment=segment,
                                        refine=refine)),
          "cos_capon_get_capon_ex")
    return [z, P, w]


@dataclass
class DeviceFrame:
    """One frame of a device call: torch CUDA tensors and parameters."""
    x: object                 # complex64 [Nx][Ny][M]
    L: int
    K: int
    d: float = 0.01
    Nb: int = 0
    z: object = None          # complex64 [Nx][Ny-2K], allocated when None
    P: object = None          # float32 [Nx][Ny-2K] or None
    w: object = None          # complex64 [Nx][Ny-2K][L] or None
    R: object = None          # complex64 [Nx][Ny-2K][L][L] or None
    V: object = None          # complex64 [Nb][L] subspace matrix or None (Butler)

    def ctypes_frame(self) -> Frame:
        Nx, Ny, M = self.x.shape
        def p(t):
            return t.data_ptr() if t is not None else None
        return Frame(p(self.x), p(self.z), p(self.P), p(self.w), p(self.R), float(self.d), int(self.L),
                     int(self.K), int(M), int(Nx), int(Ny), int(self.Nb), p(self.V))


def capon_frames(frames: Sequence[DeviceFrame], ctx: Optional[Context] = None, o: Optional[Opts] = None,
                 stream=None) -> None:
    """Run all frames in one call on `stream` (torch stream or raw handle;
    default: the current torch stream, whose handle is 0 for the default
    stream).  Asynchronous."""
    import torch
    ctx = ctx or _module_ctx()
    for f in frames:
        Nx, Ny, _M = f.x.shape
        if f.z is None:
            f.z = torch.empty((Nx, Ny - 2 * f.K), dtype=torch.complex64, device=f.x.device)
    arr = (Frame * len(frames))(*[f.ctypes_frame() for f in frames])
    if stream is None:
        stream = torch.cuda.current_stream(frames[0].x.device)
    sp = getattr(stream, "cuda_stream", stream)
    check(lib.cos_capon_run(ctx.handle, arr, len(frames), C.byref(o) if o is not None else None, sp),
          "cos_capon_run")
