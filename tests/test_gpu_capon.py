"""Parity of the CUDA Capon path (through the C ABI) with the FP64 oracle and
with outputs of the reference's own CPU path (golden fixtures).

Error measures per pixel:
  P: |P - P_ref| / P_ref                      (tolerance TOL_P, the FP32-path bar)
  z: |z - z_ref| / sqrt(P_ref)                 (amplitude error on the output's own scale)
  w: ||w - w_ref|| / ||w_ref||
"""
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL_P = 1e-4        # fused form: the 1e-4 relative output-power bar vs FP64
TOL_Z = 1e-3
TOL_W = 2e-3
# The plain FP32 form keeps the reference GPU algorithm's FP32 running sums
# along the covariance diagonals (buildR_kernel.cu:116-131); their rounding
# reaches ~2e-4 on the strongest scatterers, hence its looser bar.
TOL_P_PLAIN = 1e-3
TOL_W_PLAIN = 1e-3


def tols(form):
    return (TOL_P, TOL_Z, TOL_W) if form == 0 else (TOL_P_PLAIN, TOL_Z, TOL_W_PLAIN)
GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def cap():
    from cos_gb300 import capon
    return capon


def errors(z, P, w, ref):
    e = {"P": np.abs(P - ref["P"]) / ref["P"],
         "z": np.abs(z - ref["z"]) / np.sqrt(ref["P"])}
    if w is not None and ref.get("w") is not None:
        e["w"] = np.linalg.norm(w - ref["w"], axis=-1) / np.linalg.norm(ref["w"], axis=-1)
    return e


def assert_close(z, P, w, ref, tol_p=TOL_P, tol_z=TOL_Z, tol_w=TOL_W, what=""):
    e = errors(z, P, w, ref)
    msg = f"{what}: " + ", ".join(f"{k} max {v.max():.2e} med {np.median(v):.2e}" for k, v in e.items())
    print(msg)
    assert np.all(np.isfinite(z)) and np.all(np.isfinite(P)), msg
    assert e["P"].max() <= tol_p, msg
    assert e["z"].max() <= tol_z, msg
    if "w" in e:
        assert e["w"].max() <= tol_w, msg


@pytest.mark.parametrize("form", [0, 1])
def test_config0_slice(cap, form):
    from cos_gb300 import synth
    c = synth.config0(seed=0)
    x = np.ascontiguousarray(c["x"][:16])
    z, P, w = cap.getCaponGPU(x, c["d"], c["L"], c["K"], form=form)
    ref = oracle.capon(x, c["d"], c["L"], c["K"], nthreads=8)
    assert_close(z, P, w, ref, *tols(form), what=f"config0 form{form}")


@pytest.mark.parametrize("form", [0, 1])
def test_config1_slice(cap, form):
    from cos_gb300 import synth
    c = synth.config1(seed=1, Nx=8)
    x = c["x"]
    z, P, w = cap.getCaponGPU(x, c["d"], c["L"], c["K"], form=form)
    ref = oracle.capon(x, c["d"], c["L"], c["K"], nthreads=8)
    assert_close(z, P, w, ref, *tols(form), what=f"config1 form{form}")


@pytest.mark.parametrize("form", [0, 1])
def test_reference_golden_cases(cap, form):
    """z and w against the reference CPU path's own outputs."""
    g = np.load(os.path.join(GOLD, "capon_ref_cases.npz"))
    for i, (Nx, Ny, M, L, K, d, _seed) in enumerate(g["cases"]):
        x = g[f"x{i}"]
        z, P, w = cap.getCaponGPU(x, d, int(L), int(K), form=form)
        ref = oracle.capon(x, d, int(L), int(K))
        np.testing.assert_allclose(ref["z"], g[f"z{i}"], rtol=1e-10, atol=1e-12)
        assert_close(z, P, w, dict(ref, z=g[f"z{i}"], w=g[f"w{i}"]), *tols(form), what=f"golden case {i} form{form}")


@pytest.mark.parametrize("bs_loading", [0, 1])
@pytest.mark.parametrize("M,L,Nb", [(96, 48, 3), (128, 64, 5), (32, 16, 4), (24, 12, 7)])
def test_beamspace(cap, M, L, Nb, bs_loading):
    from cos_gb300 import synth
    x = synth.cube(96, 6, M, [10.0, 5.0], seed=M + Nb)
    V = np.zeros((Nb, L))
    z, P, w = cap.getCaponGPU(x, 0.01, L, 1, V, loading=bs_loading)
    ref = oracle.capon(x, 0.01, L, 1, Nb=Nb, bs_loading=bool(bs_loading), nthreads=6)
    assert_close(z, P, w, ref, what=f"beamspace M{M} L{L} Nb{Nb} load{bs_loading}")


def test_beamspace_full_dft_equals_element_space(cap):
    from cos_gb300 import synth
    x = synth.cube(64, 4, 24, [10.0], seed=5)
    V = np.zeros((11, 11))
    zb, Pb, wb = cap.getCaponGPU(x, 0.05, 11, 1, V)
    ref = oracle.capon(x, 0.05, 11, 1)
    assert_close(zb, Pb, wb, ref, what="beamspace Nb=L")


def test_drop_in_getCaponCUDAPy(cap):
    """[z, R, w, e] with R as the reference GPU writes it: per pixel
    column-major, loaded, not normalised (buildR_kernel.cu:84-86, 153-157)."""
    from cos_gb300 import synth
    c = synth.config0(seed=4)
    x = np.ascontiguousarray(c["x"][:2, :64])
    z, R, w, e = cap.getCaponCUDAPy(x, c["d"], c["L"], c["K"], np.array([0]), False, False)
    assert e == 0
    ref = oracle.capon(x, c["d"], c["L"], c["K"], want_R=True)
    Ns, T = x.shape[2] - c["L"] + 1, 2 * c["K"] + 1
    R_expect = np.swapaxes(ref["R"], -1, -2) * (Ns * T)   # column-major memory of R_true
    err = np.abs(R - R_expect).max() / np.abs(R_expect).max()
    assert err < 1e-5, err
    assert_close(z, ref["P"], w, ref, what="getCaponCUDAPy")


@pytest.mark.parametrize("form", [0, 1])
def test_normalised_R_output(cap, form):
    from cos_gb300 import _lib
    rng = np.random.default_rng(3)
    x = (rng.standard_normal((2, 30, 32)) + 1j * rng.standard_normal((2, 30, 32))).astype(np.complex64)
    ctx = cap.Capon()
    L, K = 16, 2
    npy = 30 - 2 * K
    z = np.zeros((2, npy), np.complex64)
    P = np.zeros((2, npy), np.float32)
    R = np.zeros((2, npy, L, L), np.complex64)
    rc = ctx.getCaponEx(z, P, None, R, x, 0.01, L, K, 32, 2, 30, 0,
                        cap.opts(form=form, r_layout=_lib.R_NORMALISED))
    assert rc == 0
    ref = oracle.capon(x, 0.01, L, K, want_R=True)
    assert np.abs(R - ref["R"]).max() / np.abs(ref["R"]).max() < 1e-5


def test_build_r_entry_point(cap):
    rng = np.random.default_rng(11)
    Nx, Nz, M, L, K = 2, 20, 24, 10, 1
    x = (rng.standard_normal((Nx, Nz, M)) + 1j * rng.standard_normal((Nx, Nz, M))).astype(np.complex64)
    R = np.zeros((Nx, Nz - 2 * K, L, L), np.complex64)
    assert cap.BuildR().getR(R, x, 0.02, L, K, M, Nx, Nz, 0) == 0
    ref = oracle.capon(x, 0.02, L, K, want_R=True)
    expect = np.swapaxes(ref["R"], -1, -2) * ((M - L + 1) * (2 * K + 1))
    assert np.abs(R - expect).max() / np.abs(expect).max() < 1e-5


def test_solver_entry_point_general_matrices(cap):
    """testRTC.pyx:183-236: general complex systems, A column-major."""
    rng = np.random.default_rng(12)
    for N, batch in ((3, 2), (16, 50), (72, 7)):
        A = (rng.standard_normal((batch, N, N)) + 1j * rng.standard_normal((batch, N, N))).astype(np.complex64)
        A += (10 * np.eye(N)).astype(np.complex64)
        b = (rng.standard_normal((batch, N)) + 1j * rng.standard_normal((batch, N))).astype(np.complex64)
        x = np.zeros((batch, N), np.complex64)
        assert cap.Solver().solve(x, A, b, N, batch) == 0
        xr = np.stack([np.linalg.solve(A[i].T.astype(np.complex128), b[i]) for i in range(batch)])
        assert np.abs(x - xr).max() / np.abs(xr).max() < 1e-4


def test_solver_known_answers(cap):
    ka = np.load(os.path.join(GOLD, "linalg_known_answers.npz"))
    for A, b, xe in ((ka["A"], ka["b1"], ka["x1"]), (ka["A"], ka["b2"], ka["x2"]),
                     (ka["complexA"], ka["complexb"], ka["complexx"])):
        Acm = np.ascontiguousarray(A.T[None].astype(np.complex64))   # column-major memory
        x = np.zeros((1, 3), np.complex64)
        assert cap.Solver().solve(x, Acm, b[None].astype(np.complex64), 3, 1) == 0
        np.testing.assert_allclose(x[0], xe, rtol=1e-5, atol=1e-6)


def test_butler_entry_point(cap):
    for Nb, L in ((3, 3), (5, 64), (3, 48), (4, 9)):
        np.testing.assert_allclose(cap.butler_matrix(Nb, L), oracle.butler(Nb, L), atol=2e-7)


@pytest.mark.parametrize("args,code", [
    (dict(L=0), 719), (dict(M=0), 719), (dict(Nx=0), 719), (dict(K=-1), 719), (dict(Nb=-1), 719),
    (dict(Nb=9), 719), (dict(L=40), 719), (dict(K=10), 719), (dict(L=65, M=80), 801),
])
def test_invalid_sizes_return_reference_codes(cap, args, code):
    """Capon.cpp:98-107 / BuildR.cpp:37-48 return cudaErrorLaunchFailure (719)."""
    a = dict(L=8, K=1, M=32, Nx=2, Nz=20, Nb=0)
    a.update(args)
    Mx = max(a["M"], 1)
    x = np.zeros((2, 20, Mx), np.complex64)
    z = np.zeros(4096, np.complex64)
    w = np.zeros(4096 * 8, np.complex64)
    rc = cap.Capon().getCapon(z, w, None, x, 0.01, a["L"], a["K"], a["M"], a["Nx"], a["Nz"], a["Nb"])
    assert rc == code


def test_multi_frame_single_call(cap):
    """Frames of different M, L, Nb in one cos_capon_run call (config-2 shapes, fewer beams)."""
    import torch
    from cos_gb300 import synth
    frames, refs = [], []
    for fr in synth.config2(seed=2, Ny=96, Nx=4):
        xt = torch.from_numpy(fr["x"]).cuda()
        Nx, Ny, M = fr["x"].shape
        npy = Ny - 2 * fr["K"]
        f = cap.DeviceFrame(x=xt, L=fr["L"], K=fr["K"], d=fr["d"], Nb=fr["Nb"],
                            P=torch.empty((Nx, npy), dtype=torch.float32, device="cuda"),
                            w=torch.empty((Nx, npy, fr["L"]), dtype=torch.complex64, device="cuda"))
        frames.append(f)
        refs.append(oracle.capon(fr["x"], fr["d"], fr["L"], fr["K"], Nb=fr["Nb"], nthreads=4))
    cap.capon_frames(frames)
    torch.cuda.synchronize()
    for f, ref in zip(frames, refs):
        assert_close(f.z.cpu().numpy(), f.P.cpu().numpy(), f.w.cpu().numpy(), ref,
                     what=f"multi-frame L{f.L} Nb{f.Nb}")


def test_full_size_config1_properties(cap):
    """Config-1 size (523,264 pixels): deterministic reruns, positive finite
    power, fused == plain within tolerance, and oracle parity on sampled beams."""
    from cos_gb300 import synth
    c = synth.config1(seed=1)
    x = c["x"]
    z1, P1, w1 = cap.getCaponGPU(x, c["d"], c["L"], c["K"], want_w=False)
    z2, P2, _ = cap.getCaponGPU(x, c["d"], c["L"], c["K"], want_w=False)
    np.testing.assert_array_equal(z1, z2)
    np.testing.assert_array_equal(P1, P2)
    assert np.all(np.isfinite(z1)) and np.all(P1 > 0)
    zp, Pp, _ = cap.getCaponGPU(x, c["d"], c["L"], c["K"], form=1, want_w=False)
    assert np.max(np.abs(Pp - P1) / P1) < TOL_P_PLAIN
    beams = [0, 97, 255]
    sub = np.ascontiguousarray(x[beams])
    ref = oracle.capon(sub, c["d"], c["L"], c["K"], want_w=False, nthreads=3)
    assert_close(z1[beams], P1[beams], None, ref, what="config1 full-size sampled beams")


# bars per case: (unrefined P, refined P, refined w).  At L=64 on the stress
# data the FP32 factorisation itself misses 1e-4 (test_oracle.py pins it with
# single-precision LAPACK on the oracle's R); the refined bar is set by the
# FP32 rounding of each range row's covariance increment.
@pytest.mark.parametrize("L,K,d,M,bars", [(64, 4, 1e-3, 128, (3e-4, 5e-5, 2e-4)),
                                          (48, 1, 0.01, 96, (TOL_P, 2e-6, 1e-4))])
def test_precise_pipeline_and_refinement(cap, L, K, d, M, bars):
    """L = 64 and 48 run the fused kernels for L > 32 (float-float covariance,
    FP32 Cholesky in registers); refine=1 adds one correction step with an
    FP64 residual inside the same kernel.  Config-3 stress case (two coherent
    scatterers one beam apart at 40 dB, loading 1e-3) for L=64."""
    from cos_gb300 import _lib, synth
    if L == 64:
        x = synth.cube(96, 3, M, [100.0, 100.0], seed=3, coherent_pair=True)
    else:
        x = synth.cube(96, 3, M, [10.0, 5.0], seed=7)
    ref = oracle.capon(x, d, L, K, nthreads=3)
    z, P, w = cap.getCaponGPU(x, d, L, K)
    assert_close(z, P, w, ref, tol_p=bars[0], what=f"fused L{L}")
    zr, Pr, wr = cap.Capon(), None, None
    Npy = x.shape[1] - 2 * K
    zr = np.zeros((3, Npy), np.complex64)
    Pr = np.zeros((3, Npy), np.float32)
    wr = np.zeros((3, Npy, L), np.complex64)
    rc = cap.Capon().getCaponEx(zr, Pr, wr, None, x, d, L, K, M, 3, x.shape[1], 0, cap.opts(refine=1))
    assert rc == 0
    e = errors(zr, Pr, wr, ref)
    print(f"refined L{L}: P max {e['P'].max():.2e}, w max {e['w'].max():.2e}")
    assert e["P"].max() <= bars[1] and e["w"].max() <= bars[2]


def test_refinement_option_on_fused_shape(cap):
    from cos_gb300 import synth
    c = synth.config1(seed=1, Nx=3, Ny=256)
    x = c["x"]
    Npy = x.shape[1] - 2 * c["K"]
    z = np.zeros((3, Npy), np.complex64)
    P = np.zeros((3, Npy), np.float32)
    assert cap.Capon().getCaponEx(z, P, None, None, x, c["d"], c["L"], c["K"], 64, 3, x.shape[1], 0,
                                  cap.opts(refine=1)) == 0
    ref = oracle.capon(x, c["d"], c["L"], c["K"], want_w=False, nthreads=3)
    assert np.max(np.abs(P - ref["P"]) / ref["P"]) <= 1e-6


def test_pinned_host_buffers_pipelined(cap):
    """Pinned host buffers take the chunked two-stream path of
    cos_capon_get_capon_ex; its outputs equal the unpinned single-chunk call."""
    import torch
    from cos_gb300 import synth
    c = synth.config1(seed=5, Nx=16, Ny=256)
    x = c["x"]
    Nx, Ny, M = x.shape
    npy = Ny - 2 * c["K"]
    ctx = cap.Capon()
    z0 = np.zeros((Nx, npy), np.complex64)
    P0 = np.zeros((Nx, npy), np.float32)
    assert ctx.getCaponEx(z0, P0, None, None, x, c["d"], c["L"], c["K"], M, Nx, Ny, 0) == 0   # tunes
    xp = torch.from_numpy(x).pin_memory()
    zp = torch.zeros((Nx, npy), dtype=torch.complex64).pin_memory()
    Pp = torch.zeros((Nx, npy), dtype=torch.float32).pin_memory()
    for _ in range(2):
        assert ctx.getCaponEx(zp.numpy(), Pp.numpy(), None, None, xp.numpy(), c["d"], c["L"], c["K"], M, Nx, Ny,
                              0) == 0
        np.testing.assert_array_equal(zp.numpy(), z0)
        np.testing.assert_array_equal(Pp.numpy(), P0)


def test_multi_frame_cuda_graph(cap):
    """The config-2 frames (uneven M, L, Nb) captured as one CUDA graph and
    replayed: the replay reproduces the eager call."""
    import torch
    from cos_gb300 import synth
    cfg = synth.config2(seed=2, Ny=64, Nx=4)
    ctx = cap.Context()
    frames = []
    for fr in cfg:
        xt = torch.from_numpy(fr["x"]).cuda()
        Nx, Ny, M = fr["x"].shape
        npy = Ny - 2 * fr["K"]
        frames.append(cap.DeviceFrame(x=xt, L=fr["L"], K=fr["K"], d=fr["d"], Nb=fr["Nb"],
                                      z=torch.empty((Nx, npy), dtype=torch.complex64, device="cuda"),
                                      P=torch.empty((Nx, npy), dtype=torch.float32, device="cuda")))
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        cap.capon_frames(frames, ctx, stream=s)            # eager: tunes, sizes buffers
    s.synchronize()
    eager = [(f.z.clone(), f.P.clone()) for f in frames]
    for f in frames:
        f.z.zero_()
        f.P.zero_()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        cap.capon_frames(frames, ctx, stream=s)
    for _ in range(2):
        g.replay()
        torch.cuda.synchronize()
        for f, (z0, P0) in zip(frames, eager):
            assert torch.equal(f.z, z0) and torch.equal(f.P, P0)


@pytest.mark.parametrize("form,tol", [(0, TOL_P), (1, TOL_P_PLAIN), (4, 1e-4)])
def test_forward_backward_averaging_element_space(cap, form, tol):
    """FB averaging (R + J R^T J)/2 against the oracle: the default form runs
    the float-float pipeline, the plain FP32 form and the TF32x3 tensor-core
    form average their own R; R output is the averaged matrix."""
    from cos_gb300 import _lib, synth
    x = synth.cube(40, 4, 64, [10.0, 5.0], seed=21)
    ref = oracle.capon(x, 0.01, 32, 2, want_R=True, fb=True, nthreads=4)
    Nx, Ny, M = x.shape
    npy = Ny - 4
    z = np.zeros((Nx, npy), np.complex64)
    P = np.zeros((Nx, npy), np.float32)
    w = np.zeros((Nx, npy, 32), np.complex64)
    R = np.zeros((Nx, npy, 32, 32), np.complex64)
    o = cap.opts(form=form, fb=1, r_layout=_lib.R_NORMALISED)
    assert cap.Capon().getCaponEx(z, P, w, R, x, 0.01, 32, 2, M, Nx, Ny, 0, o) == 0
    eP = (np.abs(P - ref["P"]) / ref["P"]).max()
    eR = np.abs(R - ref["R"]).max() / np.abs(ref["R"]).max()
    plain = oracle.capon(x, 0.01, 32, 2, nthreads=4)
    assert (np.abs(plain["P"] - ref["P"]) / ref["P"]).max() > 10 * tol   # FB changes the answer here
    print(f"form {form} fb: P {eP:.2e} R {eR:.2e}")
    assert eP < tol and eR < 1e-5
    # R is persymmetric: R[a,b] = conj(R[L-1-a, L-1-b])
    np.testing.assert_allclose(R, np.conj(R[:, :, ::-1, ::-1]), rtol=0, atol=1e-6 * np.abs(R).max())


@pytest.mark.parametrize("bs_loading", [0, 1])
@pytest.mark.parametrize("M,L,Nb", [(96, 48, 3), (128, 64, 5), (32, 16, 4)])
def test_forward_backward_averaging_beamspace(cap, M, L, Nb, bs_loading):
    from cos_gb300 import synth
    x = synth.cube(48, 4, M, [10.0, 5.0], seed=M + 3 * Nb)
    V = np.zeros((Nb, L))
    z, P, w = cap.getCaponGPU(x, 0.01, L, 1, V, doFBAvg=True, loading=bs_loading)
    ref = oracle.capon(x, 0.01, L, 1, Nb=Nb, bs_loading=bool(bs_loading), fb=True, nthreads=4)
    assert_close(z, P, w, ref, what=f"FB beamspace M{M} L{L} Nb{Nb} load{bs_loading}")


def test_forward_backward_averaging_unsupported_beams(cap):
    from cos_gb300 import _lib
    x = np.zeros((2, 20, 32), np.complex64)
    z = np.zeros((2, 18), np.complex64)
    P = np.zeros((2, 18), np.float32)
    e = cap.Capon().getCaponEx(z, P, None, None, x, 0.01, 16, 1, 32, 2, 20, 7, cap.opts(fb=1))
    assert e == _lib.ERR_NOT_SUPPORTED


@pytest.mark.parametrize("Nb", [3, 5])
def test_subspace_butler_equals_default_route(cap, Nb):
    """The Butler matrix passed as an explicit subspace (direct products) gives
    the sliding-DFT route's answer."""
    from cos_gb300 import synth
    M, L = (96, 48) if Nb == 3 else (128, 64)
    x = synth.cube(40, 4, M, [10.0, 5.0], seed=Nb + 40)
    B = cap.butler_matrix(Nb, L)
    z0, P0, w0 = cap.getCaponGPU(x, 0.01, L, 1, np.zeros((Nb, L)))
    z1, P1, w1 = cap.getCaponGPU(x, 0.01, L, 1, np.zeros((Nb, L)), subspace=B)
    assert (np.abs(P1 - P0) / P0).max() < 2e-5
    assert (np.abs(z1 - z0) / np.sqrt(P0)).max() < 1e-4


@pytest.mark.parametrize("fb", [False, True])
@pytest.mark.parametrize("bs_loading", [0, 1])
@pytest.mark.parametrize("M,L,Nb", [(32, 16, 3), (64, 32, 5)])
def test_general_subspace_matches_oracle(cap, M, L, Nb, bs_loading, fb):
    """A random (non-orthonormal) subspace: element-space loading enters as
    dl V V^H; both loadings, with and without FB averaging."""
    from cos_gb300 import synth
    rng = np.random.default_rng(M + Nb)
    V = ((rng.standard_normal((Nb, L)) + 1j * rng.standard_normal((Nb, L))) / np.sqrt(2 * L)).astype(np.complex64)
    x = synth.cube(40, 4, M, [10.0, 5.0], seed=M + 7 * Nb)
    z, P, w = cap.getCaponGPU(x, 0.01, L, 1, None, doFBAvg=fb, loading=bs_loading, subspace=V)
    ref = oracle.capon(x, 0.01, L, 1, Nb=Nb, V=V.astype(np.complex128), bs_loading=bool(bs_loading), fb=fb,
                       nthreads=4)
    assert_close(z, P, w, ref, what=f"subspace M{M} L{L} Nb{Nb} load{bs_loading} fb{int(fb)}")


def test_general_subspace_device_frame_and_limits(cap):
    import torch
    from cos_gb300 import _lib, synth
    M, L, Nb = 64, 32, 4
    rng = np.random.default_rng(3)
    V = ((rng.standard_normal((Nb, L)) + 1j * rng.standard_normal((Nb, L))) / np.sqrt(2 * L)).astype(np.complex64)
    x = synth.cube(30, 3, M, [10.0], seed=9)
    fr = cap.DeviceFrame(x=torch.from_numpy(x).cuda(), L=L, K=1, Nb=Nb, V=torch.from_numpy(V).cuda(),
                         P=torch.empty((3, 28), device="cuda"))
    cap.capon_frames([fr])
    torch.cuda.synchronize()
    ref = oracle.capon(x, 0.01, L, 1, Nb=Nb, V=V.astype(np.complex128), nthreads=3)
    assert (np.abs(fr.P.cpu().numpy() - ref["P"]) / ref["P"]).max() < TOL_P
    # a given subspace with Nb > 5 is outside the range-tile kernel
    V7 = np.ones((7, L), np.complex64)
    z = np.zeros((3, 28), np.complex64)
    P = np.zeros((3, 28), np.float32)
    e = _lib.lib.cos_capon_get_capon_subspace(cap._module_ctx().handle, z.ctypes.data, P.ctypes.data, None,
                                              x.ctypes.data, V7.ctypes.data, 0.01, L, 1, M, 3, 30, 7, None)
    assert e == _lib.ERR_NOT_SUPPORTED


def test_side_by_side_frames_equal_serial_launches():
    """A multi-frame call runs its scratch-free launch groups (fused groups,
    beamspace frames) side by side on the context's auxiliary streams; the
    outputs equal the same call with every group on the caller's stream
    (COS_CAPON_SERIAL_FRAMES=1) bit for bit, eagerly and as a graph replay."""
    import torch
    from cos_gb300 import capon, synth
    ctx = capon.Context()
    cfg = synth.config2(seed=9, Ny=160, Nx=12)

    def frames():
        out = []
        for fr in cfg:
            x = torch.from_numpy(fr["x"]).cuda()
            Nx, Ny, _ = fr["x"].shape
            f = capon.DeviceFrame(x=x, L=fr["L"], K=fr["K"], d=fr["d"], Nb=fr["Nb"])
            f.P = torch.empty((Nx, Ny - 2 * fr["K"]), dtype=torch.float32, device="cuda")
            out.append(f)
        return out

    def grab(fs):
        return [(f.z.cpu().numpy(), f.P.cpu().numpy()) for f in fs]

    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        warm = frames()
        for _ in range(2):   # tune every fused shape first: later calls fork
            capon.capon_frames(warm, ctx, stream=s)
    s.synchronize()
    os.environ["COS_CAPON_SERIAL_FRAMES"] = "1"
    try:
        ser = frames()
        with torch.cuda.stream(s):
            capon.capon_frames(ser, ctx, stream=s)
        s.synchronize()
    finally:
        del os.environ["COS_CAPON_SERIAL_FRAMES"]
    par = frames()
    with torch.cuda.stream(s):
        capon.capon_frames(par, ctx, stream=s)
    s.synchronize()
    gr = frames()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        capon.capon_frames(gr, ctx, stream=s)
    g.replay()
    torch.cuda.synchronize()
    for (za, pa), (zb, pb), (zc, pc) in zip(grab(ser), grab(par), grab(gr)):
        assert np.array_equal(za, zb) and np.array_equal(pa, pb)
        assert np.array_equal(za, zc) and np.array_equal(pa, pc)


def test_precise_pipeline_refinement_with_exact_covariance(cap):
    """The precise pipeline (R materialised in float-float with every product
    exact, FP32 Cholesky, one FP64-residual step), which the plain form with
    refine=1 and the shapes without a fused kernel take: on the L=64 stress
    data it reaches 1e-6, the accuracy the fused refinement's FP32 increments
    stop short of."""
    from cos_gb300 import _lib, synth
    x = synth.cube(96, 3, 128, [100.0, 100.0], seed=3, coherent_pair=True)
    ref = oracle.capon(x, 1e-3, 64, 4, nthreads=3)
    Npy = x.shape[1] - 8
    z = np.zeros((3, Npy), np.complex64)
    P = np.zeros((3, Npy), np.float32)
    w = np.zeros((3, Npy, 64), np.complex64)
    o = cap.opts(form=_lib.FORM_PLAIN, refine=_lib.REFINE_ALL)
    assert cap.Capon().getCaponEx(z, P, w, None, x, 1e-3, 64, 4, 128, 3, x.shape[1], 0, o) == 0
    e = errors(z, P, w, ref)
    print(f"precise refined L64: P max {e['P'].max():.2e}, w max {e['w'].max():.2e}")
    assert e["P"].max() <= 1e-6 and e["w"].max() <= 1e-5
