"""Adjoint of the output power: the torch.linalg reference gradient is checked
against FP64 central finite differences on CPU; the CUDA adjoint
(cos_capon_backward behind capon_power) is checked against that reference."""
import math

import numpy as np
import pytest
import torch

from cos_gb300.autograd import capon_power_reference


def _case(seed, Nx=2, Ny=24, M=16, dtype=torch.complex128):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((Nx, Ny, M)) + 1j * rng.standard_normal((Nx, Ny, M))
    x += 3.0 * np.exp(1j * 0.6 * np.arange(M))
    return torch.tensor(x, dtype=dtype)


def test_reference_gradient_matches_fp64_finite_differences():
    L, K, f0 = 8, 1, 0.25
    x = _case(1).requires_grad_(True)
    delta = torch.tensor(0.7, dtype=torch.float64, requires_grad=True)
    tau = torch.tensor(np.random.default_rng(2).uniform(-0.05, 0.05, 16), requires_grad=True)
    loss = capon_power_reference(x, delta, tau, L, K, f0).sum()
    loss.backward()
    h = 1e-6

    def f(xx=None, dd=None, tt=None):
        with torch.no_grad():
            return capon_power_reference(x if xx is None else xx, delta if dd is None else dd,
                                         tau if tt is None else tt, L, K, f0).sum().item()

    fd = (f(dd=delta + h) - f(dd=delta - h)) / (2 * h)
    assert abs(fd - delta.grad.item()) <= 1e-6 * max(1.0, abs(fd))
    for m in (0, 7, 15):
        e = torch.zeros(16, dtype=torch.float64)
        e[m] = h
        fd = (f(tt=tau + e) - f(tt=tau - e)) / (2 * h)
        assert abs(fd - tau.grad[m].item()) <= 1e-6 * max(1.0, abs(fd))
    for (b, y, m) in ((0, 5, 3), (1, 12, 9), (0, 20, 15)):
        for unit in (1.0, 1j):
            e = torch.zeros_like(x.detach())
            e[b, y, m] = h * unit
            fd = (f(xx=x.detach() + e) - f(xx=x.detach() - e)) / (2 * h)
            g = x.grad[b, y, m]
            # torch's complex gradient is 2 dl/dconj(x): dl = Re(conj(g) dx)
            expect = (g.real if unit == 1.0 else g.imag).item()
            assert abs(fd - expect) <= 1e-6 * max(1.0, abs(fd)), (b, y, m, unit, fd, expect)


@pytest.mark.gpu
@pytest.mark.parametrize("L,K,M,Ny", [(32, 2, 64, 48), (16, 1, 32, 40), (8, 1, 16, 30)])
def test_cuda_adjoint_matches_reference_gradient(L, K, M, Ny):
    from cos_gb300.autograd import capon_power
    f0 = 0.25
    rng = np.random.default_rng(L)
    x64 = _case(L, Nx=3, Ny=Ny, M=M)
    tau0 = rng.uniform(-0.05, 0.05, M)
    # reference loading: 0.01 tr(R)/L of the data, as an absolute scalar
    delta0 = 0.01 * float(torch.mean(torch.sum(torch.abs(x64) ** 2, -1)).item()) * 1.0
    mask = torch.tensor(rng.random((3, Ny - 2 * K)) < 0.5, dtype=torch.float64)

    xr = x64.clone().requires_grad_(True)
    dr = torch.tensor(delta0, dtype=torch.float64, requires_grad=True)
    tr = torch.tensor(tau0, requires_grad=True)
    Pr = capon_power_reference(xr, dr, tr, L, K, f0).reshape(3, Ny - 2 * K)
    (Pr * mask).sum().backward()

    xg = x64.to(torch.complex64).cuda().requires_grad_(True)
    dg = torch.tensor(delta0, dtype=torch.float32, device="cuda", requires_grad=True)
    tg = torch.tensor(tau0, dtype=torch.float32, device="cuda", requires_grad=True)
    Pg = capon_power(xg, dg, tg, L, K, f0)
    (Pg * mask.to(torch.float32).cuda()).sum().backward()

    relP = (torch.abs(Pg.detach().cpu().double() - Pr.detach()) / Pr.detach()).max().item()
    assert relP < 1e-4, relP
    gx_err = (torch.abs(xg.grad.cpu().to(torch.complex128) - xr.grad).max() / torch.abs(xr.grad).max()).item()
    gd_err = abs(dg.grad.item() - dr.grad.item()) / abs(dr.grad.item())
    gt_err = (torch.abs(tg.grad.cpu().double() - tr.grad).max() / torch.abs(tr.grad).max()).item()
    print(f"L{L}: P {relP:.2e} grad x {gx_err:.2e} delta {gd_err:.2e} tau {gt_err:.2e}")
    assert gx_err < 1e-3 and gd_err < 1e-3 and gt_err < 1e-3


def _pixel_losses(x, delta, tau, L, K, f0, b, p):
    """FP64 output power of the listed (beam, pixel) pairs (torch.linalg)."""
    return capon_power_reference(x, delta, tau, L, K, f0, pixels=(b, p))


@pytest.mark.gpu
def test_config4_gradients_full_frame():
    """The differentiation workload as specified: the config-1 batch
    [Nx=256][Ny=2048][M=64], L=32, K=2, delays tau_m ~ U(-0.05, 0.05) applied as
    exp(-j 2 pi f0 tau_m) with f0 = 0.25, a learnable absolute loading delta
    initialised at 0.01 tr(R)/L, loss = sum of P over a seeded 64 x 64 pixel
    mask.  The CUDA gradients are checked against FP64 central differences
    (step 1e-6) for 256 random input samples inside the mask's support, and
    against torch.linalg autograd for delta and tau."""
    from cos_gb300 import synth
    from cos_gb300.autograd import capon_power
    L, K, f0 = 32, 2, 0.25
    c = synth.config1(seed=4)
    x = c["x"]
    Nx, Ny, M = x.shape
    rng = np.random.default_rng(4)
    tau0 = rng.uniform(-0.05, 0.05, M)
    # 0.01 tr(R)/L of the normalised covariance = 0.01 * mean snapshot energy per element
    delta0 = 0.01 * float(np.mean(np.abs(x.astype(np.complex128)) ** 2))
    b0, p0 = int(rng.integers(0, Nx - 64)), int(rng.integers(0, Ny - 2 * K - 64))
    mask = np.zeros((Nx, Ny - 2 * K))
    mask[b0:b0 + 64, p0:p0 + 64] = 1.0

    xg = torch.from_numpy(x).cuda().requires_grad_(True)
    dg = torch.tensor(delta0, dtype=torch.float32, device="cuda", requires_grad=True)
    tg = torch.tensor(tau0, dtype=torch.float32, device="cuda", requires_grad=True)
    Pg = capon_power(xg, dg, tg, L, K, f0)
    (Pg * torch.from_numpy(mask).float().cuda()).sum().backward()
    gx = xg.grad.cpu().numpy()

    # torch.linalg reference over the mask (FP64)
    bb, pp = np.nonzero(mask)
    bt, pt = torch.from_numpy(bb), torch.from_numpy(pp)
    x64 = torch.from_numpy(x.astype(np.complex128))
    dr = torch.tensor(delta0, dtype=torch.float64, requires_grad=True)
    tr = torch.tensor(tau0, requires_grad=True)
    _pixel_losses(x64, dr, tr, L, K, f0, bt, pt).sum().backward()
    gd_err = abs(dg.grad.item() - dr.grad.item()) / abs(dr.grad.item())
    gt_err = (torch.abs(tg.grad.cpu().double() - tr.grad).max() / torch.abs(tr.grad).max()).item()

    # FP64 central differences for 256 random input samples under the mask
    h = 1e-6
    errs = []
    scale = np.abs(gx[b0:b0 + 64, p0:p0 + 64 + 2 * K]).max()
    for _ in range(256):
        b = b0 + int(rng.integers(0, 64))
        y = p0 + int(rng.integers(0, 64 + 2 * K))
        m = int(rng.integers(0, M))
        unit = 1.0 if rng.random() < 0.5 else 1j
        # pixels of beam b whose window contains row y and lie in the mask
        ps = np.arange(max(p0, y - 2 * K), min(p0 + 64, y + 1))
        if ps.size == 0:
            continue
        # only beam b's rows ps[0] .. ps[-1] + 2K enter these pixels
        r0 = int(ps[0])
        sub = x64[b:b + 1, r0:int(ps[-1]) + 2 * K + 1]
        bsel, psel = torch.zeros(ps.size, dtype=torch.long), torch.from_numpy(ps - r0)
        xp, xm = sub.clone(), sub.clone()
        xp[0, y - r0, m] += h * unit
        xm[0, y - r0, m] -= h * unit
        with torch.no_grad():
            fd = (_pixel_losses(xp, dr, tr, L, K, f0, bsel, psel).sum() -
                  _pixel_losses(xm, dr, tr, L, K, f0, bsel, psel).sum()).item() / (2 * h)
        g = gx[b, y, m]
        expect = g.real if unit == 1.0 else g.imag
        errs.append(abs(fd - expect) / scale)
    print(f"config 4: delta {gd_err:.2e} tau {gt_err:.2e} x (FD, {len(errs)} samples, max rel to scale) "
          f"{max(errs):.2e}")
    assert len(errs) >= 200
    assert gd_err < 1e-3 and gt_err < 1e-3 and max(errs) < 1e-3
