"""Parity of the tensor-core fused form (COS_CAPON_FORM_TC_FUSED: the Hankel
Gram per range row on tcgen05 with an FP16 hi/lo split, the window sum and the
register Cholesky on chip) with the FP64 oracle, through the C ABI.

The bar is the fused form's: P within 1e-4 relative of FP64, z within 1e-3 of
sqrt(P).  Shapes: the three instantiations (L, 2K+1, M) = (32, 5, 64),
(32, 3, 64), (16, 3, 32); partial last tiles; one-pixel beams; frames batched
into one launch; rows whose amplitudes differ by many orders of magnitude
(each row is scaled by its own power of two before the FP16 split, and the
sliding window sum restarts where a leaving row would cancel small ones).
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL_P = 1e-4
TOL_Z = 1e-3


def run_tcf(x, L, K, d, loading=0, form=None):
    import torch
    from cos_gb300 import _lib, capon
    f = capon.DeviceFrame(x=torch.from_numpy(np.ascontiguousarray(x)).cuda(), L=L, K=K, d=d)
    Nx, Ny, _ = x.shape
    f.z = torch.empty((Nx, Ny - 2 * K), dtype=torch.complex64, device="cuda")
    f.P = torch.empty((Nx, Ny - 2 * K), dtype=torch.float32, device="cuda")
    capon.capon_frames([f], o=capon.opts(form=_lib.FORM_TC_FUSED if form is None else form, loading=loading))
    torch.cuda.synchronize()
    return f.z.cpu().numpy(), f.P.cpu().numpy()


def check(z, P, ref, what):
    eP = np.abs(P - ref["P"]) / ref["P"]
    ez = np.abs(z - ref["z"]) / np.sqrt(ref["P"])
    msg = f"{what}: P max {eP.max():.2e} med {np.median(eP):.2e}, z max {ez.max():.2e}"
    print(msg)
    assert np.all(np.isfinite(P)) and np.all(np.isfinite(z)), msg
    assert eP.max() <= TOL_P and ez.max() <= TOL_Z, msg


def test_config1_slice():
    from cos_gb300 import synth
    c = synth.config1(seed=1, Nx=8)
    z, P = run_tcf(c["x"], c["L"], c["K"], c["d"])
    check(z, P, oracle.capon(c["x"], c["d"], c["L"], c["K"], want_w=False, nthreads=8), "config1 tc-fused")


def test_config0_shape():
    from cos_gb300 import synth
    c = synth.config0(seed=0)
    x = np.ascontiguousarray(c["x"][:16])
    z, P = run_tcf(x, c["L"], c["K"], c["d"])
    check(z, P, oracle.capon(x, c["d"], c["L"], c["K"], want_w=False, nthreads=8), "config0 tc-fused")


def test_config2_element_frame():
    from cos_gb300 import synth
    fr = [f for f in synth.config2(seed=2) if f["L"] == 32 and f["Nb"] == 0][0]
    x = np.ascontiguousarray(fr["x"][:6])
    z, P = run_tcf(x, fr["L"], fr["K"], fr["d"])
    check(z, P, oracle.capon(x, fr["d"], fr["L"], fr["K"], want_w=False, nthreads=6), "config2 (64,32) tc-fused")


@pytest.mark.parametrize("Ny", [5, 6, 37, 99, 164])
def test_partial_tiles(Ny):
    """Ny - 2K pixels per beam not a multiple of the 16-pixel unit, down to one pixel."""
    from cos_gb300 import synth
    if Ny >= 32:
        x = synth.cube(Ny, 3, 64, [10.0, 4.0], seed=Ny)
    else:   # too short for the generator's scatterer envelope: noise only
        rng = np.random.default_rng(Ny)
        x = (rng.standard_normal((3, Ny, 64)) + 1j * rng.standard_normal((3, Ny, 64))).astype(np.complex64)
    z, P = run_tcf(x, 32, 2, 0.01)
    check(z, P, oracle.capon(x, 0.01, 32, 2, want_w=False), f"Ny={Ny}")


def test_absolute_loading():
    from cos_gb300 import synth
    x = synth.cube(130, 3, 64, [10.0], seed=7)
    z, P = run_tcf(x, 32, 2, 0.05, loading=2)
    check(z, P, oracle.capon(x, 0.05, 32, 2, want_w=False, absolute=True, fp32_scalars=False), "absolute loading")


def test_rows_of_very_different_amplitude():
    """Each row's own power-of-two scale keeps the FP16 split at 22 bits, and
    the window sum restarts instead of subtracting a row that dwarfs the rest."""
    from cos_gb300 import synth
    x = synth.cube(100, 3, 64, [10.0], seed=11)
    rng = np.random.default_rng(5)
    x = (x * (10.0 ** rng.uniform(-6, 3, size=(1, 100, 1)))).astype(np.complex64)
    z, P = run_tcf(x, 32, 2, 0.01)
    check(z, P, oracle.capon(x, 0.01, 32, 2, want_w=False), "row amplitudes 1e-6..1e3")


def test_batched_frames_equal_single_calls():
    import torch
    from cos_gb300 import _lib, capon, synth
    xs = [synth.cube(90 + 7 * i, 3 + i, 64, [10.0], seed=20 + i) for i in range(3)]
    singles = [run_tcf(x, 32, 2, 0.01) for x in xs]
    frames = []
    for x in xs:
        f = capon.DeviceFrame(x=torch.from_numpy(x).cuda(), L=32, K=2, d=0.01)
        f.P = torch.empty((x.shape[0], x.shape[1] - 4), dtype=torch.float32, device="cuda")
        frames.append(f)
    capon.capon_frames(frames, o=capon.opts(form=_lib.FORM_TC_FUSED))
    torch.cuda.synchronize()
    for f, (z, P) in zip(frames, singles):
        assert np.array_equal(f.P.cpu().numpy(), P) and np.array_equal(f.z.cpu().numpy(), z)


def test_repeatable_and_close_to_fp32_fused():
    from cos_gb300 import synth
    c = synth.config1(seed=3, Nx=4)
    z1, P1 = run_tcf(c["x"], c["L"], c["K"], c["d"])
    z2, P2 = run_tcf(c["x"], c["L"], c["K"], c["d"])
    assert np.array_equal(P1, P2) and np.array_equal(z1, z2)
    zf, Pf = run_tcf(c["x"], c["L"], c["K"], c["d"], form=0)
    assert np.max(np.abs(P1 - Pf) / Pf) < 1e-4


def test_unsupported_requests_are_refused():
    import torch
    from cos_gb300 import _lib, capon, synth
    x = torch.from_numpy(synth.cube(40, 2, 64, [10.0], seed=1)).cuda()
    f = capon.DeviceFrame(x=x, L=32, K=2, d=0.01)
    f.w = torch.empty((2, 36, 32), dtype=torch.complex64, device="cuda")
    with pytest.raises(_lib.CaponError) as ei:
        capon.capon_frames([f], o=capon.opts(form=_lib.FORM_TC_FUSED))
    assert ei.value.status == _lib.ERR_NOT_SUPPORTED
    g = capon.DeviceFrame(x=x, L=24, K=2, d=0.01)   # no instantiation for L = 24
    with pytest.raises(_lib.CaponError) as ei:
        capon.capon_frames([g], o=capon.opts(form=_lib.FORM_TC_FUSED))
    assert ei.value.status == _lib.ERR_NOT_SUPPORTED
