"""Drop-in equivalence with the reference's own GPU library.

RealTimeCapon is built from its sources (oracle/build_rtc.py; skipped where
they are not staged) and run through Capon::getCapon beside this project's
drop-in entry points on the same inputs:
  * R: the memory the reference copies back (per pixel column-major, loaded,
    not normalised) against cos_capon_build_r / getCaponCUDAPy's R;
  * z and w against getCaponCUDAPy (both FP32; the reference's sliding
    covariance rounding bounds the agreement);
  * the error codes for invalid sizes.
"""
import ctypes
import os
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.join(os.path.dirname(HERE), "oracle")


@pytest.fixture(scope="module")
def rtc():
    import build_rtc
    if not os.path.isdir(build_rtc.SRC) and not os.path.isdir(os.path.join(build_rtc.REF, "framework")):
        pytest.skip("reference RealTimeCapon sources not staged")
    lib = ctypes.CDLL(build_rtc.build())
    vp, fl, i = ctypes.c_void_p, ctypes.c_float, ctypes.c_int
    lib.rtc_get_capon.argtypes = [vp, vp, vp, vp, fl, i, i, i, i, i, i]
    return lib


def _run_rtc(lib, x, d, L, K, Nb=0):
    Nx, Ny, M = x.shape
    npy = Ny - 2 * K
    z = np.zeros((Nx, npy), np.complex64)
    w = np.zeros((Nx, npy, L), np.complex64)
    R = np.zeros((Nx, npy, L, L), np.complex64)
    cwd = os.getcwd()
    os.chdir(tempfile.mkdtemp(prefix="rtc_"))   # the library writes its timer files here
    try:
        e = lib.rtc_get_capon(z.ctypes.data, w.ctypes.data, R.ctypes.data, x.ctypes.data, d, L, K, M, Nx, Ny, Nb)
    finally:
        os.chdir(cwd)
    return e, z, w, R


@pytest.mark.parametrize("M,L,K", [(64, 32, 2), (32, 16, 1)])
def test_drop_in_matches_reference_gpu_library(rtc, M, L, K):
    from cos_gb300 import capon, synth
    x = synth.cube(48, 4, M, [10.0, 5.0], seed=M + K)
    e, z_r, w_r, R_r = _run_rtc(rtc, x, 0.01, L, K)
    assert e == 0
    z, R, w, e2 = capon.getCaponCUDAPy(x, 0.01, L, K, None)
    assert e2 == 0
    scale = np.abs(R_r).max()
    eR = np.abs(R - R_r).max() / scale
    ez = (np.abs(z - z_r) / np.abs(z_r).max()).max()
    ew = (np.linalg.norm(w - w_r, axis=-1) / np.linalg.norm(w_r, axis=-1)).max()
    print(f"M{M} L{L} K{K}: R {eR:.2e} z {ez:.2e} w {ew:.2e}")
    # same memory layout and convention; both FP32 (the reference slides its
    # diagonal sums, this build telescopes them), so agreement to FP32 rounding of R
    assert eR < 2e-6
    assert ez < 1e-3 and ew < 5e-3


def test_error_codes_match_reference_gpu_library(rtc):
    """Sizes the reference rejects at the top of Capon::getCapon
    (Capon.cpp:98-107), before any allocation or launch: Nb > L, Nx < 1."""
    from cos_gb300 import capon
    x = np.zeros((2, 20, 16), np.complex64)
    z = np.zeros((2, 18), np.complex64)
    w = np.zeros((2, 18, 8), np.complex64)
    R = np.zeros((2, 18, 8, 8), np.complex64)
    cwd = os.getcwd()
    os.chdir(tempfile.mkdtemp(prefix="rtc_"))
    try:
        for (Nx, Nb) in [(2, 9), (0, 0)]:
            e = rtc.rtc_get_capon(z.ctypes.data, w.ctypes.data, R.ctypes.data, x.ctypes.data, 0.01, 8, 1, 16, Nx,
                                  20, Nb)
            ours = capon.Capon().getCapon(z, w, None, x, 0.01, 8, 1, 16, Nx, 20, Nb)
            assert e == ours == 719, (Nx, Nb, e, ours)
    finally:
        os.chdir(cwd)


@pytest.mark.parametrize("M,L,Nb", [(32, 16, 3), (64, 32, 5)])
def test_beamspace_against_reference_gpu_library(rtc, M, L, Nb):
    """The reference's default beamspace route (Butler matrix, three batched
    cuBLAS GEMMs around an Nb x Nb solve, Capon.cpp:285-417) on the same cube:
    both are held against the FP64 oracle, this build to the fused tolerance,
    and the two agree to within the reference's own FP32 error."""
    import oracle
    from cos_gb300 import capon, synth
    K = 1
    x = synth.cube(40, 4, M, [10.0, 5.0], seed=M + Nb)
    e, z_r, w_r, _ = _run_rtc(rtc, x, 0.01, L, K, Nb)
    assert e == 0
    z, R, w, e2 = capon.getCaponCUDAPy(x, 0.01, L, K, np.zeros((Nb, L)), want_R=False)
    assert e2 == 0
    ref = oracle.capon(x, 0.01, L, K, Nb=Nb, nthreads=4)
    sP = np.sqrt(ref["P"])
    ez_ours = (np.abs(z - ref["z"]) / sP).max()
    ez_rtc = (np.abs(z_r - ref["z"]) / sP).max()
    ew_ours = (np.linalg.norm(w - ref["w"], axis=-1) / np.linalg.norm(ref["w"], axis=-1)).max()
    ew_rtc = (np.linalg.norm(w_r - ref["w"], axis=-1) / np.linalg.norm(ref["w"], axis=-1)).max()
    print(f"M{M} L{L} Nb{Nb}: z ours {ez_ours:.2e} ref-lib {ez_rtc:.2e}; w ours {ew_ours:.2e} ref-lib {ew_rtc:.2e}")
    assert ez_ours < 1e-3 and ew_ours < 2e-3
    assert ez_rtc < 1e-2 and ew_rtc < 5e-2
    assert (np.abs(z - z_r) / sP).max() < 2 * ez_rtc + 1e-3


def test_build_r_against_reference_gpu_library(rtc):
    """IBuildR::getR (element space): the same R memory (column-major, loaded,
    not normalised) from the reference library and cos_capon_build_r."""
    from cos_gb300 import capon, synth
    vp, fl, i = ctypes.c_void_p, ctypes.c_float, ctypes.c_int
    rtc.rtc_build_r.argtypes = [vp, vp, fl, i, i, i, i, i, i]
    M, L, K = 64, 32, 2
    x = synth.cube(40, 3, M, [10.0], seed=7)
    Nx, Ny, _ = x.shape
    R_r = np.zeros((Nx, Ny - 2 * K, L, L), np.complex64)
    assert rtc.rtc_build_r(R_r.ctypes.data, x.ctypes.data, 0.01, L, K, M, Nx, Ny, 0) == 0
    R = np.zeros_like(R_r)
    assert capon.BuildR().getR(R, x, 0.01, L, K, M, Nx, Ny, 0) == 0
    e = np.abs(R - R_r).max() / np.abs(R_r).max()
    print(f"build_r vs reference library: {e:.2e}")
    assert e < 2e-6


@pytest.mark.parametrize("N", [1, 3, 5, 11, 32, 72])
def test_solver_against_reference_gpu_library(rtc, N):
    """ISolver::solve: general complex systems (column-major A), the
    reference's batched pivoted LU (nvidia_solve.cu) against cos_capon_solve."""
    from cos_gb300 import capon
    vp, i = ctypes.c_void_p, ctypes.c_int
    rtc.rtc_solve.argtypes = [vp, vp, vp, i, i]
    rng = np.random.default_rng(N)
    batch = 64
    A = (rng.standard_normal((batch, N, N)) + 1j * rng.standard_normal((batch, N, N))) / np.sqrt(N)
    A += 2.0 * np.eye(N)                                     # well conditioned, not Hermitian
    b = rng.standard_normal((batch, N)) + 1j * rng.standard_normal((batch, N))
    Acm = np.ascontiguousarray(np.transpose(A, (0, 2, 1))).astype(np.complex64)   # column-major per system
    b32 = b.astype(np.complex64)
    x_r = np.zeros((batch, N), np.complex64)
    assert rtc.rtc_solve(x_r.ctypes.data, Acm.ctypes.data, b32.ctypes.data, N, batch) == 0
    x = np.zeros((batch, N), np.complex64)
    assert capon.Solver().solve(x, Acm, b32, N, batch) == 0
    ref = np.linalg.solve(A, b[..., None])[..., 0]
    e_ours = (np.linalg.norm(x - ref, axis=1) / np.linalg.norm(ref, axis=1)).max()
    e_lib = (np.linalg.norm(x_r - ref, axis=1) / np.linalg.norm(ref, axis=1)).max()
    print(f"N={N}: ours {e_ours:.2e} reference library {e_lib:.2e}")
    assert e_ours < 1e-5 and e_lib < 1e-4
