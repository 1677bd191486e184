"""Parity of the fused element-space kernels for L > 32 (capon_fused_wide.cuh:
the covariance in float-float, built and factored block by block in
registers) with the FP64 oracle, through the C ABI.

The refinement option (opts.refine = 1) runs inside the same kernel: the
float-float covariance slots are kept in a per-warp stash, the residual
a - R x0 is formed with exact products and float-float sums (assembled in
FP64), and one correction solve reuses the register factor.

Shapes: the config-3 precision stress case (M=128, L=64, K=4, two coherent
scatterers one beam apart at 40 dB, loading 1e-3) and L=48, K=1 at M=96.  The
bar is the fused form's: P within 1e-4 relative of FP64, z within 1e-3 of
sqrt(P); w and R are checked where the mode writes them.  Also: partial range
tiles, a channel count without a compile-time instantiation, absolute
loading, frames batched into one launch.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL_P = 1e-4
TOL_Z = 1e-3
# the precision stress slice: FP32 factorisation of R rounded once already
# misses 1e-4 on its worst pixels (pinned on the CPU in test_oracle.py)
TOL_P_STRESS = 2e-4


def run(x, L, K, d, loading=0, want_w=False, want_R=False, refine=0):
    import torch
    from cos_gb300 import _lib, capon
    Nx, Ny, M = x.shape
    npy = Ny - 2 * K
    f = capon.DeviceFrame(x=torch.from_numpy(np.ascontiguousarray(x)).cuda(), L=L, K=K, d=d)
    f.z = torch.empty((Nx, npy), dtype=torch.complex64, device="cuda")
    f.P = torch.empty((Nx, npy), dtype=torch.float32, device="cuda")
    if want_w:
        f.w = torch.empty((Nx, npy, L), dtype=torch.complex64, device="cuda")
    if want_R:
        f.R = torch.empty((Nx, npy, L, L), dtype=torch.complex64, device="cuda")
    capon.capon_frames([f], o=capon.opts(form=_lib.FORM_FUSED, loading=loading, r_layout=_lib.R_NORMALISED,
                                         refine=refine))
    torch.cuda.synchronize()
    out = {"z": f.z.cpu().numpy(), "P": f.P.cpu().numpy()}
    if want_w:
        out["w"] = f.w.cpu().numpy()
    if want_R:
        out["R"] = f.R.cpu().numpy()
    return out


def check(o, ref, what, tol_p=TOL_P):
    eP = np.abs(o["P"] - ref["P"]) / ref["P"]
    ez = np.abs(o["z"] - ref["z"]) / np.sqrt(ref["P"])
    msg = f"{what}: P max {eP.max():.2e} med {np.median(eP):.2e}, z max {ez.max():.2e}"
    if "w" in o:
        ew = np.linalg.norm(o["w"] - ref["w"], axis=-1) / np.linalg.norm(ref["w"], axis=-1)
        msg += f", w max {ew.max():.2e}"
    print(msg)
    assert np.all(np.isfinite(o["P"])) and np.all(np.isfinite(o["z"])), msg
    assert eP.max() <= tol_p and ez.max() <= TOL_Z, msg
    return msg


def config3_slice(Nx=3, Ny=200, seed=3):
    """A small cube from the config-3 generator (the coherent pair, 40 dB)."""
    from cos_gb300 import synth
    x = synth.cube(Ny, Nx, 128, [100.0, 100.0], seed=seed, coherent_pair=True)
    return x, dict(L=64, K=4, d=1e-3)


def test_config3_beams_z_p_w():
    """The coherent pair's beams: z/P from the z/P kernel, w from the w kernel."""
    x, c = config3_slice()
    ref = oracle.capon(x, c["d"], c["L"], c["K"], nthreads=3)
    check(run(x, c["L"], c["K"], c["d"]), ref, "config3 fused L64 z/P", TOL_P_STRESS)
    o = run(x, c["L"], c["K"], c["d"], want_w=True)
    msg = check(o, ref, "config3 fused L64 w mode", TOL_P_STRESS)
    ew = np.linalg.norm(o["w"] - ref["w"], axis=-1) / np.linalg.norm(ref["w"], axis=-1)
    assert ew.max() <= 2e-3, msg


def test_config3_loaded_covariance():
    """R mode: the loaded, normalised covariance against the oracle's, per pixel
    max|dR| / max|R| (float-float covariance rounded once to FP32)."""
    x, c = config3_slice(Nx=2, Ny=80)
    ref = oracle.capon(x, c["d"], c["L"], c["K"], want_R=True, nthreads=2)
    o = run(x, c["L"], c["K"], c["d"], want_R=True)
    npy = x.shape[1] - 2 * c["K"]
    eR = (np.abs(o["R"] - ref["R"]).reshape(2, npy, -1).max(-1)
          / np.abs(ref["R"]).reshape(2, npy, -1).max(-1))
    print(f"config3 R: max {eR.max():.2e} med {np.median(eR):.2e}")
    assert eR.max() <= 4e-7


def test_l48_k1():
    from cos_gb300 import synth
    x = synth.cube(150, 3, 96, [10.0, 5.0], seed=7)
    ref = oracle.capon(x, 0.01, 48, 1, nthreads=3)
    check(run(x, 48, 1, 0.01), ref, "L48 K1 z/P")
    o = run(x, 48, 1, 0.01, want_w=True)
    check(o, ref, "L48 K1 w mode")


@pytest.mark.parametrize("Ny", [9, 10, 31, 57])
def test_partial_tiles(Ny):
    """Ny - 2K pixels per beam not a multiple of the 16-pixel tile, down to one."""
    rng = np.random.default_rng(Ny)
    x = (rng.standard_normal((2, Ny, 128)) + 1j * rng.standard_normal((2, Ny, 128))).astype(np.complex64)
    ref = oracle.capon(x, 0.01, 64, 4, want_w=False)
    check(run(x, 64, 4, 0.01), ref, f"L64 Ny={Ny}")


def test_channel_count_without_instantiation():
    """M = 100 has no compile-time instantiation: the run-time-M candidate."""
    from cos_gb300 import synth
    x = synth.cube(60, 2, 100, [10.0], seed=9)
    ref = oracle.capon(x, 0.01, 64, 4, want_w=False)
    check(run(x, 64, 4, 0.01), ref, "L64 M100")


def test_absolute_loading():
    from cos_gb300 import synth
    x = synth.cube(60, 2, 128, [10.0], seed=4)
    ref = oracle.capon(x, 0.05, 64, 4, want_w=False, absolute=True, fp32_scalars=False)
    check(run(x, 64, 4, 0.05, loading=2), ref, "L64 absolute loading")


def test_batched_frames_equal_single_calls():
    import torch
    from cos_gb300 import capon, synth
    xs = [synth.cube(40 + 9 * i, 2 + i, 128, [10.0], seed=30 + i) for i in range(3)]
    singles = [run(x, 64, 4, 0.01) for x in xs]
    frames = []
    for x in xs:
        f = capon.DeviceFrame(x=torch.from_numpy(x).cuda(), L=64, K=4, d=0.01)
        f.P = torch.empty((x.shape[0], x.shape[1] - 8), dtype=torch.float32, device="cuda")
        frames.append(f)
    capon.capon_frames(frames)
    torch.cuda.synchronize()
    for f, s in zip(frames, singles):
        assert np.array_equal(f.P.cpu().numpy(), s["P"]) and np.array_equal(f.z.cpu().numpy(), s["z"])


def test_refinement_config3():
    """One refinement step inside the fused kernel: the stress slice's worst
    pixels come within the 1e-4 bar that the FP32 factorisation misses.  What
    is left is the FP32 rounding of each range row's covariance increment,
    which the float-float R inherits."""
    x, c = config3_slice()
    ref = oracle.capon(x, c["d"], c["L"], c["K"], nthreads=3)
    o = run(x, c["L"], c["K"], c["d"], want_w=True, refine=1)
    msg = check(o, ref, "config3 fused L64 refined")
    eP = np.abs(o["P"] - ref["P"]) / ref["P"]
    ew = np.linalg.norm(o["w"] - ref["w"], axis=-1) / np.linalg.norm(ref["w"], axis=-1)
    assert eP.max() <= 5e-5 and ew.max() <= 1e-4, msg
    o2 = run(x, c["L"], c["K"], c["d"], refine=1)   # z and P only: the same numbers
    assert np.array_equal(o2["P"], o["P"]) and np.array_equal(o2["z"], o["z"])


def test_refinement_l48_and_loaded_covariance():
    from cos_gb300 import synth
    x = synth.cube(80, 2, 96, [10.0, 5.0], seed=8)
    ref = oracle.capon(x, 0.01, 48, 1, want_R=True, nthreads=2)
    o = run(x, 48, 1, 0.01, want_w=True, want_R=True, refine=1)
    check(o, ref, "L48 refined")
    eP = np.abs(o["P"] - ref["P"]) / ref["P"]
    assert eP.max() <= 1e-6
    npy = x.shape[1] - 2
    eR = (np.abs(o["R"] - ref["R"]).reshape(2, npy, -1).max(-1)
          / np.abs(ref["R"]).reshape(2, npy, -1).max(-1))
    assert eR.max() <= 4e-7


def test_adaptive_refinement_refines_only_ill_conditioned_pixels():
    """opts.refine = 2: a pixel's outputs are either the plain fused form's,
    bit for bit (pivot spread <= 32), or the refine-all form's (the pixels
    above it; within 1e-6, the refinement pass forming its first covariance
    row from the pixel's own rows, not the tile's), and the refined ones are
    few.  The result meets the refined bar on the stress slice."""
    from cos_gb300 import _lib
    x, c = config3_slice()
    ref = oracle.capon(x, c["d"], c["L"], c["K"], want_w=False, nthreads=3)
    o0 = run(x, c["L"], c["K"], c["d"])
    o1 = run(x, c["L"], c["K"], c["d"], refine=_lib.REFINE_ALL)
    o2 = run(x, c["L"], c["K"], c["d"], refine=_lib.REFINE_ADAPTIVE)
    plain = (o2["P"] == o0["P"]) & (o2["z"] == o0["z"])
    close = np.abs(o2["P"] - o1["P"]) <= 1e-6 * o1["P"]
    assert np.all(plain | close)
    frac = 1.0 - plain.mean()
    msg = check(o2, ref, f"config3 fused L64 adaptive ({frac:.1%} refined)")
    assert 0 < frac < 0.3, msg
    eP = np.abs(o2["P"] - ref["P"]) / ref["P"]
    assert eP.max() <= 5e-5, msg


@pytest.mark.parametrize("L,K,M", [(64, 1, 128), (64, 2, 96), (64, 0, 80), (64, 2, 101), (48, 2, 96), (48, 4, 64),
                                   (48, 0, 80)])
def test_other_temporal_windows(L, K, M):
    """The L > 32 instantiations take the window 2K+1 from the frame: any K
    whose tile fits in shared memory runs the fused kernel (z/P, w, and the
    adaptive refinement).  M = 101: range rows not 16-byte aligned, staged
    with plain loads instead of the bulk copy."""
    from cos_gb300 import _lib, synth
    x = synth.cube(70, 3, M, [10.0, 4.0], seed=L + K + M)
    ref = oracle.capon(x, 0.01, L, K, nthreads=3)
    check(run(x, L, K, 0.01), ref, f"L{L} K{K} M{M} z/P")
    o = run(x, L, K, 0.01, want_w=True)
    msg = check(o, ref, f"L{L} K{K} M{M} w mode")
    ew = np.linalg.norm(o["w"] - ref["w"], axis=-1) / np.linalg.norm(ref["w"], axis=-1)
    assert ew.max() <= 2e-3, msg
    check(run(x, L, K, 0.01, refine=_lib.REFINE_ADAPTIVE), ref, f"L{L} K{K} M{M} adaptive")


@pytest.mark.parametrize("refine", [0, 2])
def test_graph_replay_equals_eager_call(refine):
    """A frame of the L > 32 kernels (z/P, and the adaptive refinement whose
    pass uses the context's stash) captured into a CUDA graph after a warm
    call: each replay writes the eager call's outputs bit for bit."""
    import torch
    from cos_gb300 import _lib, capon
    x, c = config3_slice(Nx=2, Ny=120)
    xt = torch.from_numpy(x).cuda()
    ctx = capon.Context()
    o = capon.opts(form=_lib.FORM_FUSED, refine=refine)

    def frame():
        f = capon.DeviceFrame(x=xt, L=c["L"], K=c["K"], d=c["d"])
        f.P = torch.empty((2, 120 - 2 * c["K"]), dtype=torch.float32, device="cuda")
        return f

    s = torch.cuda.Stream()
    eager = frame()
    with torch.cuda.stream(s):
        for _ in range(2):   # tunes the shape and sizes the stash
            capon.capon_frames([eager], ctx, o, stream=s)
    s.synchronize()
    gf = frame()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        capon.capon_frames([gf], ctx, o, stream=s)
    for _ in range(2):
        gf.P.zero_()
        g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(gf.P.cpu().numpy(), eager.P.cpu().numpy())
        assert np.array_equal(gf.z.cpu().numpy(), eager.z.cpu().numpy())


def test_refinement_at_l32():
    """L = 32 (config-1 shape): refinement on every pixel and the adaptive
    mode run in the fused path, through the one-warp-per-pixel instantiation
    of the blocked path; z/P without refinement stays with the L = 32
    kernel."""
    from cos_gb300 import _lib, synth
    c = synth.config1(seed=1, Nx=4, Ny=300)
    x = c["x"]
    ref = oracle.capon(x, c["d"], c["L"], c["K"], nthreads=4)
    o1 = run(x, c["L"], c["K"], c["d"], want_w=True, refine=_lib.REFINE_ALL)
    msg = check(o1, ref, "L32 refined")
    eP = np.abs(o1["P"] - ref["P"]) / ref["P"]
    ew = np.linalg.norm(o1["w"] - ref["w"], axis=-1) / np.linalg.norm(ref["w"], axis=-1)
    assert eP.max() <= 1e-6 and ew.max() <= 1e-5, msg
    o0 = run(x, c["L"], c["K"], c["d"])
    o2 = run(x, c["L"], c["K"], c["d"], refine=_lib.REFINE_ADAPTIVE)
    check(o2, ref, "L32 adaptive")
    # config-1 data is well conditioned: the adaptive mode's first pass (the
    # blocked path's z/P, not the L = 32 kernel's) decides for most pixels
    plain = o2["P"] != o1["P"]
    assert plain.mean() > 0.5


def test_refinement_at_l16():
    """L = 16 (config-0 shape): refinement in the fused path through the
    16-lanes-per-pixel instantiation of the blocked path."""
    from cos_gb300 import _lib, synth
    c = synth.config0(seed=0)
    x = np.ascontiguousarray(c["x"][:6])
    ref = oracle.capon(x, c["d"], c["L"], c["K"], nthreads=6)
    o1 = run(x, c["L"], c["K"], c["d"], want_w=True, refine=_lib.REFINE_ALL)
    msg = check(o1, ref, "L16 refined")
    eP = np.abs(o1["P"] - ref["P"]) / ref["P"]
    ew = np.linalg.norm(o1["w"] - ref["w"], axis=-1) / np.linalg.norm(ref["w"], axis=-1)
    assert eP.max() <= 1e-6 and ew.max() <= 1e-5, msg
    check(run(x, c["L"], c["K"], c["d"], refine=_lib.REFINE_ADAPTIVE), ref, "L16 adaptive")


def test_refinement_in_a_multi_frame_call_equals_single_calls():
    """One call with an L=32 and an L=64 frame and refinement: the groups
    share the context's stash one after the other; each frame's outputs equal
    its own single-frame call bit for bit."""
    import torch
    from cos_gb300 import _lib, capon, synth
    a = synth.config1(seed=4, Nx=2, Ny=90)["x"]
    b, _ = config3_slice(Nx=2, Ny=90)
    shapes = [(a, 32, 2, 0.01), (b, 64, 4, 1e-3)]
    o = capon.opts(form=_lib.FORM_FUSED, refine=_lib.REFINE_ALL)
    ctx = capon.Context()

    def frame(x, L, K, d):
        f = capon.DeviceFrame(x=torch.from_numpy(x).cuda(), L=L, K=K, d=d)
        f.P = torch.empty((x.shape[0], x.shape[1] - 2 * K), dtype=torch.float32, device="cuda")
        return f

    singles = []
    for sh in shapes:
        f = frame(*sh)
        capon.capon_frames([f], ctx, o)
        singles.append(f)
    both = [frame(*sh) for sh in shapes]
    capon.capon_frames(both, ctx, o)
    torch.cuda.synchronize()
    for f, g in zip(both, singles):
        assert np.array_equal(f.P.cpu().numpy(), g.P.cpu().numpy())
        assert np.array_equal(f.z.cpu().numpy(), g.z.cpu().numpy())


def _sweep_cases(n, seed):
    rng = np.random.default_rng(seed)
    cases = []
    for _ in range(n):
        L = int(rng.choice([16, 32, 48, 64]))
        K = int(rng.integers(0, 5 if L > 32 else 3))
        M = int(rng.integers(L + 16, min(L + 80, 150) + 1))
        Ny = int(rng.integers(2 * K + 1, 90))
        Nx = int(rng.integers(1, 4))
        refine = int(rng.integers(0, 3))
        loading = int(rng.choice([0, 2]))
        cases.append((L, K, M, Ny, Nx, refine, loading, int(rng.integers(1 << 30))))
    return cases


@pytest.mark.parametrize("L,K,M,Ny,Nx,refine,loading,seed", _sweep_cases(10, 2024))
def test_random_shapes(L, K, M, Ny, Nx, refine, loading, seed):
    """Seeded random shapes through the fused path: L = 48 and 64 (z/P and
    refinement) and the refinement modes at L = 16 and 32; odd and even M,
    short beams, both loading conventions."""
    if L <= 32 and refine == 0:
        refine = 1   # the L <= 32 kernels' own z/P is covered elsewhere
    if (M - L + 1) * (2 * K + 1) < 2 * L and refine == 0:
        refine = 1   # fewer snapshots than 2L: an ill-conditioned R, FP32-limited
    rng = np.random.default_rng(seed)
    x = (rng.standard_normal((Nx, Ny, M)) + 1j * rng.standard_normal((Nx, Ny, M))).astype(np.complex64)
    x[:, Ny // 2] *= 8.0   # one strong range row
    d = 0.05 if loading == 2 else 0.01
    ref = oracle.capon(x, d, L, K, want_w=False, absolute=loading == 2, fp32_scalars=loading != 2)
    o = run(x, L, K, d, loading=loading, refine=refine)
    check(o, ref, f"L{L} K{K} M{M} Ny{Ny} Nx{Nx} refine{refine} load{loading}")
