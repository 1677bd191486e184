"""Edge shapes of the element-space Capon path against the FP64 oracle.

Each case exercises a branch the config-sized tests do not reach:
  * odd M, so a beam's range rows are not 16-byte aligned and the fused
    kernel reads the cube with plain loads instead of the bulk copy;
  * K = 0 (one range sample per pixel, the T = 1 instantiations);
  * a single pixel per beam (Ny = 2K + 1) and a single beam;
  * a range count one pixel past a whole tile, so the last tile of each beam
    holds one pixel;
  * an M without a compile-time instantiation (run-time M);
  * L = M, one subarray (Ns = 1), where R has rank <= 2K + 1 before loading;
  * an M whose tile would not fit in shared memory (the frame takes the
    precise pipeline instead of the fused kernel).
Both the fused form (0) and the plain three-stage form (1) run every case.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL_P = {0: 1e-4, 1: 1e-3}   # fused: the 1e-4 power bar; plain: its FP32 running sums
TOL_Z = 1e-3
TOL_W = 2e-3

# (Nx, Ny, M, L, K, d, what)
CASES = [
    (3, 41, 33, 16, 1, 0.01, "odd M, unaligned rows"),
    (2, 37, 17, 16, 0, 0.01, "odd M, K=0"),
    (2, 70, 64, 32, 0, 0.01, "L=32, K=0"),
    (1, 5, 40, 16, 2, 0.01, "one beam, one pixel"),
    (2, 69, 64, 32, 2, 0.01, "one pixel past a whole tile"),
    (2, 90, 48, 32, 1, 0.01, "run-time M"),
    (2, 30, 16, 16, 1, 0.1, "L = M, one subarray"),
    (2, 40, 96, 32, 2, 0.01, "M past the fused tile's shared memory"),
]


def _cube(Nx, Ny, M, seed):
    rng = np.random.default_rng(seed)
    x = (rng.standard_normal((Nx, Ny, M)) + 1j * rng.standard_normal((Nx, Ny, M))) / np.sqrt(2.0)
    # one plane wave across the channels on every beam, so R is not white
    ph = np.exp(1j * np.pi * 0.37 * np.arange(M))
    env = 4.0 * np.exp(-0.5 * ((np.arange(Ny) - Ny / 2) / 4.0) ** 2)
    x += env[None, :, None] * ph[None, None, :]
    return x.astype(np.complex64)


@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("Nx,Ny,M,L,K,d,what", CASES, ids=[c[-1] for c in CASES])
def test_edge_shape_matches_oracle(form, Nx, Ny, M, L, K, d, what):
    from cos_gb300 import capon
    x = _cube(Nx, Ny, M, seed=Nx * 1000 + Ny * 10 + M)
    z, P, w = capon.getCaponGPU(x, d, L, K, form=form)
    ref = oracle.capon(x, d, L, K, nthreads=2)
    assert z.shape == (Nx, Ny - 2 * K) and w.shape == (Nx, Ny - 2 * K, L)
    eP = np.abs(P - ref["P"]) / ref["P"]
    ez = np.abs(z - ref["z"]) / np.sqrt(ref["P"])
    ew = np.linalg.norm(w - ref["w"], axis=-1) / np.linalg.norm(ref["w"], axis=-1)
    msg = f"{what} form{form}: P {eP.max():.2e}, z {ez.max():.2e}, w {ew.max():.2e}"
    print(msg)
    assert np.all(np.isfinite(z)) and np.all(np.isfinite(P)) and np.all(np.isfinite(w)), msg
    assert eP.max() <= TOL_P[form], msg
    assert ez.max() <= TOL_Z, msg
    assert ew.max() <= TOL_W, msg


@pytest.mark.parametrize("form", [0, 1])
def test_outputs_do_not_depend_on_the_batch(form):
    """A beam's outputs are the same whether it runs alone or inside a larger
    frame (no cross-beam or cross-tile leakage through the staged rows)."""
    from cos_gb300 import capon
    x = _cube(5, 133, 64, seed=7)
    z, P, w = capon.getCaponGPU(x, 0.01, 32, 2, form=form)
    for b in (0, 3, 4):
        zb, Pb, wb = capon.getCaponGPU(np.ascontiguousarray(x[b:b + 1]), 0.01, 32, 2, form=form)
        np.testing.assert_array_equal(zb[0], z[b])
        np.testing.assert_array_equal(Pb[0], P[b])
        np.testing.assert_array_equal(wb[0], w[b])


def test_mixed_outputs_in_one_fused_group():
    """Frames of equal (L, K, M) share one fused launch per output mode: R,
    when any frame asks for it, comes from its own covariance pass, and z, P
    (and w) from the factorising launch.  Each frame's outputs must equal
    those of a call that is given that frame alone: bit for bit, except z of
    a frame without w, which the group's w-mode launch forms from x = R^-1 a
    (z = x^H g / a^H R^-1 a) and a z/P launch from the carried L^-1 g."""
    import torch
    from cos_gb300 import capon
    L, K, M, Nx, Ny = 32, 2, 64, 3, 150
    npy = Ny - 2 * K
    xs = [torch.from_numpy(_cube(Nx, Ny, M, seed=30 + i)).cuda() for i in range(4)]
    want = [(True, False), (False, True), (True, True), (False, False)]   # (w, R)

    def make(x, w, R):
        return capon.DeviceFrame(
            x=x, L=L, K=K, d=0.01,
            P=torch.empty((Nx, npy), dtype=torch.float32, device="cuda"),
            w=torch.empty((Nx, npy, L), dtype=torch.complex64, device="cuda") if w else None,
            R=torch.empty((Nx, npy, L, L), dtype=torch.complex64, device="cuda") if R else None)

    ctx = capon.Context()
    group = [make(x, w, R) for x, (w, R) in zip(xs, want)]
    capon.capon_frames(group, ctx)
    torch.cuda.synchronize()
    for f, x, (w, R) in zip(group, xs, want):
        alone = make(x, w, R)
        capon.capon_frames([alone], ctx)
        torch.cuda.synchronize()
        assert torch.equal(alone.P, f.P)
        if w:
            assert torch.equal(alone.z, f.z)
        else:
            scale = torch.sqrt(f.P)
            assert float((torch.abs(alone.z - f.z) / scale).max()) < 1e-5
        if w:
            assert torch.equal(alone.w, f.w)
        if R:
            assert torch.equal(alone.R, f.R)
            assert bool(torch.isfinite(torch.view_as_real(f.R)).all())
