"""cos_capon_run_plain_noalloc: the allocation-free entry point.

Callers that cannot allocate device memory (code running inside another
framework's allocator, real-time loops that must not reach the driver's
allocator) get a variant of the plain FP32 pipeline whose work buffers live in
a fixed file-scope device array.  This test calls it through the C ABI and
checks its outputs against the context-based entry point on the same inputs,
for two calls in a row with different data (the array keeps the previous
call's contents, so stale state would show), and checks that a frame too large
for the array is refused.  The file name sorts last so that a run that stops at
the first failure has run every other test before this one.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_P = 1e-6   # same kernels and arithmetic as the context path: results agree to rounding
TOL_Z = 1e-6


def _frame(lib, x, z, P, w, L, K, d=0.01):
    Nx, Ny, M = x.shape
    return lib.Frame(x.data_ptr(), z.data_ptr(), P.data_ptr(), w.data_ptr(), None, float(d), L, K, M, Nx, Ny, 0)


def _outputs(torch, Nx, npy, L):
    return (torch.empty((Nx, npy), dtype=torch.complex64, device="cuda"),
            torch.empty((Nx, npy), dtype=torch.float32, device="cuda"),
            torch.empty((Nx, npy, L), dtype=torch.complex64, device="cuda"))


def test_noalloc_matches_context_path_twice():
    import torch
    from cos_gb300 import _lib, capon, synth

    L, K = 16, 1
    for call, seed in enumerate((21, 22)):
        x = torch.from_numpy(synth.cube(200, 4, 32, [10.0, 5.0], seed=seed)).cuda()
        Nx, Ny, M = x.shape
        npy = Ny - 2 * K
        z, P, w = _outputs(torch, Nx, npy, L)
        fr = _frame(_lib, x, z, P, w, L, K)
        rc = _lib.lib.cos_capon_run_plain_noalloc(C.byref(fr), None)
        assert rc == 0, _lib.status_string(rc)
        torch.cuda.synchronize()

        ref = capon.DeviceFrame(x=x, L=L, K=K, d=0.01)
        ref.z, ref.P, ref.w = _outputs(torch, Nx, npy, L)
        capon.capon_frames([ref], o=capon.opts(form=_lib.FORM_PLAIN))
        torch.cuda.synchronize()

        Pn, Pr = P.cpu().numpy(), ref.P.cpu().numpy()
        zn, zr = z.cpu().numpy(), ref.z.cpu().numpy()
        wn, wr = w.cpu().numpy(), ref.w.cpu().numpy()
        assert np.all(np.isfinite(Pn)) and np.all(Pn > 0), f"call {call}"
        assert np.max(np.abs(Pn - Pr) / Pr) <= TOL_P, f"call {call}"
        assert np.max(np.abs(zn - zr) / np.sqrt(Pr)) <= TOL_Z, f"call {call}"
        assert np.max(np.abs(wn - wr)) <= 1e-5 * np.max(np.abs(wr)), f"call {call}"


def test_noalloc_refuses_frames_beyond_its_array():
    import torch
    from cos_gb300 import _lib

    L, K = 32, 2
    x = torch.zeros((8, 1024, 64), dtype=torch.complex64, device="cuda")   # 8*1020*(32*32+32) > 2^20
    z, P, w = _outputs(torch, 8, 1020, L)
    fr = _frame(_lib, x, z, P, w, L, K)
    assert _lib.lib.cos_capon_run_plain_noalloc(C.byref(fr), None) == _lib.ERR_OUT_OF_MEMORY
    fr.L = 0
    assert _lib.lib.cos_capon_run_plain_noalloc(C.byref(fr), None) == _lib.ERR_LAUNCH
