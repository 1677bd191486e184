"""Time-domain steering: the oracle against the reference's own interpolation
(scipy interp1d, as tdibC.pyx:47-49 calls it) and analytic known answers on
CPU; the CUDA kernel against the oracle, and steering -> Capon against the
oracle chain, on the GPU."""
import numpy as np
import pytest

import tdib_oracle


def _scipy_steer(s):
    """tdibC.pyx:9-67 line by line with scipy.interpolate.interp1d."""
    interpolate = pytest.importorskip("scipy.interpolate")
    mf, t = s["mfdata"].astype(np.complex128), s["mtaxe"]
    xx, zz = np.mean(s["x_r"]) / 2, np.mean(s["D"]) / 2
    n_x, n_y = s["xarr"].shape
    out = np.zeros((n_x, n_y, mf.shape[0]), complex)
    for nx in range(n_x):
        r_t = np.sqrt((xx + s["xarr"][nx]) ** 2 + s["yarr"][nx] ** 2 + zz ** 2)
        for n in range(mf.shape[0]):
            r_r = np.sqrt((xx + s["xarr"][nx] - s["x_r"][n]) ** 2 + s["yarr"][nx] ** 2 + (zz - s["D"][n]) ** 2)
            tipos = (r_t + r_r) * (1.0 / s["c"])
            re = interpolate.interp1d(t, mf[n].real, kind="linear", bounds_error=False)(tipos)
            im = interpolate.interp1d(t, mf[n].imag, kind="linear", bounds_error=False)(tipos)
            out[nx, :, n] = (re + 1j * im) * np.exp(2j * np.pi * s["fc"] * tipos)
    return out


def test_oracle_matches_reference_interpolation():
    s = tdib_oracle.scenario(seed=1, n_h=6, n_s=400, n_x=3, n_y=40)
    s["yarr"][:, -3:] = 400.0   # a few pixels beyond the time axis: NaN in both
    a = tdib_oracle.steer(**s)
    b = _scipy_steer(s)
    assert np.array_equal(np.isnan(a), np.isnan(b)) and np.isnan(a).any()
    m = ~np.isnan(a)
    # the two interpolation formulas round differently (~1e-11 of the data scale)
    np.testing.assert_allclose(a[m], b[m], rtol=1e-10, atol=1e-10)
    img = tdib_oracle.tdib(**s)
    assert img.shape == (40, 3)
    np.testing.assert_allclose(img[~np.isnan(img)], (b.sum(2).T / 6)[~np.isnan(img)], rtol=1e-10, atol=1e-10)


def test_oracle_known_answer():
    """One hydrophone at the origin's mirror point: tau = 2 r / c exactly, a
    linear ramp in time interpolates exactly, fc = 0 leaves it unmixed."""
    c, dt = 1500.0, 1e-4
    t = np.arange(1000) * dt
    mf = (t * 10.0 + 1j * (5.0 - t)).astype(np.complex128)[None, :]
    x_r, D = np.array([0.0]), np.array([0.0])
    yarr = np.array([[3.0, 7.5, 80.0]])
    xarr = np.zeros_like(yarr)
    Xd = tdib_oracle.steer(mf, t, x_r, D, c, 0.0, xarr, yarr)
    tau = 2 * yarr[0] / c
    np.testing.assert_allclose(Xd[0, :2, 0], (tau * 10.0 + 1j * (5.0 - tau))[:2], rtol=1e-12)
    assert np.isnan(Xd[0, 2, 0])                 # 0.1067 s is past the 0.0999 s axis


@pytest.mark.gpu
def test_cuda_steering_matches_oracle():
    from cos_gb300 import tdib
    s = tdib_oracle.scenario(seed=2, n_h=24, n_s=3000, n_x=6, n_y=256)
    s["yarr"][:, -5:] = 2000.0
    ref = tdib_oracle.steer(**s)
    Xd = tdib.steer(**s)
    img = tdib.tdib(**s)
    assert np.array_equal(np.isnan(Xd), np.isnan(ref))
    m = ~np.isnan(ref)
    err = np.abs(Xd[m] - ref[m]).max() / np.abs(ref[m]).max()
    ref_img = tdib_oracle.tdib(**s)
    mi = ~np.isnan(ref_img)
    err_img = np.abs(img[mi] - ref_img[mi]).max() / np.abs(ref_img[mi]).max()
    print(f"steer {err:.2e} image {err_img:.2e}")
    # FP32 per-hydrophone delay corrections on an FP64 per-pixel base: the
    # carrier phase to ~3e-6 rad, the sample index to ~5e-7
    assert err < 1e-5 and err_img < 1e-5


@pytest.mark.gpu
def test_steering_then_capon_matches_oracle_chain():
    import oracle
    from cos_gb300 import capon, tdib
    s = tdib_oracle.scenario(seed=3, n_h=32, n_s=2048, n_x=4, n_y=200)
    Xd = tdib.steer(**s)
    assert not np.isnan(Xd).any()
    z, P, w = capon.getCaponGPU(Xd, 0.01, 16, 1)
    ref = oracle.capon(tdib_oracle.steer(**s).astype(np.complex64), 0.01, 16, 1)
    relP = (np.abs(P - ref["P"]) / ref["P"]).max()
    print(f"steer -> capon P {relP:.2e}")
    assert relP < 1e-4


def test_oracle_matches_reference_tdibC():
    """The oracle against runs of the reference's own tdibC.tdib
    (tdibC.pyx:9-67, executed by tests/golden/make_golden.py with its
    numpy/print shims), NaN placement included."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "tdib_ref_cases.npz"))
    keys = ("mfdata", "mtaxe", "x_r", "D", "c", "fc", "xarr", "yarr")
    for i in range(int(g["ncases"])):
        s = {k: g[f"{k}{i}"] for k in keys}
        s["c"], s["fc"] = float(s["c"]), float(s["fc"])
        img = tdib_oracle.tdib(**s)
        ref = g[f"image{i}"]
        assert np.array_equal(np.isnan(img), np.isnan(ref))
        m = ~np.isnan(ref)
        np.testing.assert_allclose(img[m], ref[m], rtol=1e-10, atol=1e-10 * np.abs(ref[m]).max())
