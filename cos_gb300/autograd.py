"""Differentiable Capon output power (torch.autograd.Function over the C ABI).

    P = capon_power(x, delta, tau, L, K, f0)

x      complex64 [Nx][Ny][M] on a CUDA device (pre-steered channel data)
delta  0-dim float32 tensor: absolute diagonal loading on the normalised
       covariance, R_d = R + delta I (learnable)
tau    float32 [M]: per-element steering delays in samples, applied as the
       phase exp(-j 2 pi f0 tau_m) (learnable)
P      float32 [Nx][Ny-2K]: MVDR output power per pixel

The forward runs the CUDA path with the weights w saved; the backward is the
hand-written adjoint kernel (cos_capon_backward), which needs only x' (the
phased cube) and w because dP = w^H dR_d w.  PyTorch's complex-gradient
convention (grad = 2 dl/dconj(x)) is applied here.
"""
from __future__ import annotations

import ctypes as C
import math

import torch

from . import _lib, capon


class _CaponPower(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, delta, tau, L, K, f0, cctx):
        Nx, Ny, M = x.shape
        npy = Ny - 2 * K
        theta = (2.0 * math.pi * f0) * tau.to(torch.float32)
        phase = torch.polar(torch.ones_like(theta), -theta).to(torch.complex64)
        xp = (x * phase).contiguous()
        fr = capon.DeviceFrame(x=xp, L=L, K=K, d=float(delta), Nb=0,
                               z=torch.empty((Nx, npy), dtype=torch.complex64, device=x.device),
                               P=torch.empty((Nx, npy), dtype=torch.float32, device=x.device),
                               w=torch.empty((Nx, npy, L), dtype=torch.complex64, device=x.device))
        capon.capon_frames([fr], cctx, capon.opts(loading=_lib.LOAD_ABSOLUTE))
        ctx.save_for_backward(xp, fr.w, phase)
        ctx.meta = (L, K, f0, cctx)
        return fr.P

    @staticmethod
    def backward(ctx, gP):
        xp, w, phase = ctx.saved_tensors
        L, K, f0, cctx = ctx.meta
        Nx, Ny, M = xp.shape
        gP = gP.contiguous().to(torch.float32)
        gx = torch.zeros_like(xp)
        gd = torch.zeros(1, dtype=torch.float32, device=xp.device)
        gth = torch.zeros(M, dtype=torch.float32, device=xp.device)
        adj = _lib.Adjoint(xp.data_ptr(), w.data_ptr(), gP.data_ptr(), gx.data_ptr(), gd.data_ptr(),
                           gth.data_ptr(), L, K, M, Nx, Ny)
        stream = torch.cuda.current_stream(xp.device).cuda_stream
        _lib.check(_lib.lib.cos_capon_backward((cctx or capon._module_ctx()).handle, C.byref(adj), stream),
                   "cos_capon_backward")
        grad_x = 2.0 * torch.conj(phase) * gx          # x' = phase * x
        grad_delta = gd[0]
        grad_tau = (2.0 * math.pi * f0) * gth          # theta = 2 pi f0 tau
        return grad_x, grad_delta, grad_tau, None, None, None, None


def capon_power(x, delta, tau, L, K, f0=0.25, ctx=None):
    """MVDR power per pixel, differentiable in x, delta and tau."""
    return _CaponPower.apply(x, delta, tau, L, K, f0, ctx)


def capon_power_reference(x, delta, tau, L, K, f0=0.25, pixels=None):
    """The same power in plain torch (complex128, torch.linalg), differentiable
    by autograd; `pixels` = optional (beam, pixel) index tensors to evaluate."""
    xp = x * torch.polar(torch.ones_like(tau), -(2.0 * math.pi * f0) * tau)
    Nx, Ny, M = x.shape
    T, Ns = 2 * K + 1, M - L + 1
    if pixels is None:
        b = torch.arange(Nx).repeat_interleave(Ny - 2 * K)
        p = torch.arange(Ny - 2 * K).repeat(Nx)
    else:
        b, p = pixels
    win = torch.stack([xp[b, p + t] for t in range(T)], 1)            # [n, T, M]
    sub = win.unfold(2, L, 1)                                          # [n, T, Ns, L]
    sub = sub.reshape(sub.shape[0], T * Ns, L)
    R = torch.einsum("nqi,nqj->nij", sub, sub.conj()) / (Ns * T)
    R = R + delta * torch.eye(L, dtype=R.dtype, device=R.device)
    a = torch.ones(R.shape[0], L, 1, dtype=R.dtype, device=R.device)
    Ria = torch.linalg.solve(R, a)
    return 1.0 / torch.real(torch.sum(Ria[..., 0], -1))
