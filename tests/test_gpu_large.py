"""A frame past 2^31 channel samples on the fused path.

The reference's host code sizes its buffers with `int` products (for example
L*L*Npx in Capon.cpp), so a cube of more than 2^31 complex samples is where
32-bit index arithmetic would wrap.  Here the cube is [4096][8192][64]
(2^31 samples, 17 GB), generated on the device.  The last beam starts past
element 2^31; its outputs must equal, bit for bit, those of a call that is
given that beam alone (each pixel's arithmetic depends only on its own range
tile), and every output must be finite and positive.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_cube_past_2_to_the_31_samples():
    torch = pytest.importorskip("torch")
    from cos_gb300 import capon
    Nx, Ny, M, L, K = 4096, 8192, 64, 32, 2
    need = Nx * Ny * M * 8 + 2 * Nx * (Ny - 2 * K) * 12
    free, _total = torch.cuda.mem_get_info()
    if free < need + (4 << 30):
        pytest.skip(f"needs {need / 2**30:.1f} GiB of free device memory")
    g = torch.Generator(device="cuda").manual_seed(5)
    x = torch.randn((Nx, Ny, M), dtype=torch.complex64, device="cuda", generator=g)
    assert x.numel() >= 2**31
    f = capon.DeviceFrame(x=x, L=L, K=K, d=0.01,
                          P=torch.empty((Nx, Ny - 2 * K), dtype=torch.float32, device="cuda"))
    capon.capon_frames([f])
    torch.cuda.synchronize()
    P = f.P
    assert bool(torch.isfinite(P).all()) and bool((P > 0).all())
    assert bool(torch.isfinite(torch.view_as_real(f.z)).all())
    for b in (Nx - 1, Nx // 2):
        fb = capon.DeviceFrame(x=x[b:b + 1], L=L, K=K, d=0.01,
                               P=torch.empty((1, Ny - 2 * K), dtype=torch.float32, device="cuda"))
        capon.capon_frames([fb])
        torch.cuda.synchronize()
        np.testing.assert_array_equal(fb.P.cpu().numpy()[0], P[b].cpu().numpy())
        np.testing.assert_array_equal(fb.z.cpu().numpy()[0], f.z[b].cpu().numpy())
    del x, f
    torch.cuda.empty_cache()
