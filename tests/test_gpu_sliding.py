"""Sliding-window inverse form (COS_CAPON_FORM_SLIDING_INVERSE) against the
FP64 oracle that follows the same rank-1 change sequence
(getCaponAllC.pyx:240-252, woodburyc.pyx:15-107), through the C ABI.

FP32 Sherman-Morrison changes lose accuracy as the window's covariance becomes
ill-conditioned (strong scatterers over small absolute loading): downdates
remove large terms by cancellation.  The tolerances below are those of each
case's conditioning, measured by an FP32 emulation of the same sequence."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cap():
    from cos_gb300 import capon
    return capon


def _run(cap, x, d, L, K, seg):
    from cos_gb300 import _lib
    return cap.getCaponGPU(x, d, L, K, form=_lib.FORM_SLIDING_INVERSE, loading=_lib.LOAD_ABSOLUTE, segment=seg)


def _err(z, P, w, ref):
    eP = np.abs(P - ref["P"]) / ref["P"]
    ez = np.abs(z - ref["z"]) / np.sqrt(ref["P"])
    ew = np.linalg.norm(w - ref["w"], axis=-1) / np.linalg.norm(ref["w"], axis=-1)
    return eP, ez, ew


def _white(seed, Nx, Ny, M, amp=2.0):
    rng = np.random.default_rng(seed)
    x = ((rng.standard_normal((Nx, Ny, M)) + 1j * rng.standard_normal((Nx, Ny, M))) / np.sqrt(2)).astype(np.complex64)
    return x + (amp * np.exp(1j * 0.3 * np.arange(M))).astype(np.complex64)


@pytest.mark.parametrize("seg", [1, 8, 64])
def test_config0_shape_matches_oracle(cap, seg):
    from cos_gb300 import synth
    x = np.ascontiguousarray(synth.config0()["x"][:6, :200])
    z, P, w = _run(cap, x, 1.0, 16, 1, seg)
    ref = oracle.capon_sliding(x, 1.0, 16, 1, seg, nthreads=6)
    eP, ez, ew = _err(z, P, w, ref)
    print(f"seg {seg}: P {eP.max():.2e} z {ez.max():.2e} w {ew.max():.2e}")
    assert eP.max() < 1e-5 and ez.max() < 1e-4 and ew.max() < 1e-4


@pytest.mark.parametrize("seg", [8, 64])
def test_l32_well_conditioned_matches_oracle(cap, seg):
    x = _white(41, 4, 300, 64)
    z, P, w = _run(cap, x, 0.5, 32, 2, seg)
    ref = oracle.capon_sliding(x, 0.5, 32, 2, seg, nthreads=4)
    eP, ez, ew = _err(z, P, w, ref)
    print(f"seg {seg}: P {eP.max():.2e} z {ez.max():.2e} w {ew.max():.2e}")
    assert eP.max() < 2e-5 and ez.max() < 1e-4 and ew.max() < 1e-4


def test_sliding_equals_direct_solve_when_well_conditioned(cap):
    # the tracked inverse and the fused Cholesky path give the same Capon
    # outputs under the same absolute loading
    from cos_gb300 import _lib
    x = _white(42, 4, 260, 64)
    zs, Ps, ws = _run(cap, x, 0.5, 32, 2, 16)
    zf, Pf, wf = cap.getCaponGPU(x, 0.5, 32, 2, loading=_lib.LOAD_ABSOLUTE)
    assert np.max(np.abs(Ps - Pf) / Pf) < 3e-5
    assert np.max(np.abs(zs - zf) / np.sqrt(Pf)) < 1e-4


def test_config1_shape_drift_is_bounded(cap):
    # 20 dB scatterers, loading 1.0: FP32 downdates drift; the median stays
    # near FP32 rounding and the worst pixel within a few 1e-3
    from cos_gb300 import synth
    x = synth.config1(Nx=4, Ny=200)["x"]
    z, P, w = _run(cap, x, 1.0, 32, 2, 8)
    ref = oracle.capon_sliding(x, 1.0, 32, 2, 8, nthreads=4)
    eP = np.abs(P - ref["P"]) / ref["P"]
    print(f"config1 shape: P max {eP.max():.2e} median {np.median(eP):.2e}")
    assert np.all(np.isfinite(P))
    assert np.median(eP) < 1e-5 and eP.max() < 2e-2


def test_options_outside_the_form(cap):
    from cos_gb300 import _lib
    x = _white(43, 2, 40, 32)
    F, A = _lib.FORM_SLIDING_INVERSE, _lib.LOAD_ABSOLUTE
    with pytest.raises(_lib.CaponError) as e:        # relative loading
        cap.getCaponGPU(x, 0.5, 16, 1, form=F)
    assert e.value.status == _lib.ERR_NOT_SUPPORTED
    with pytest.raises(_lib.CaponError) as e:        # beamspace
        cap.getCaponGPU(x, 0.5, 16, 1, np.zeros((3, 16)), form=F, loading=A)
    assert e.value.status == _lib.ERR_NOT_SUPPORTED
    with pytest.raises(_lib.CaponError) as e:        # L > 32
        cap.getCaponGPU(_white(44, 1, 20, 64), 0.5, 48, 1, form=F, loading=A)
    assert e.value.status == _lib.ERR_NOT_SUPPORTED
    with pytest.raises(_lib.CaponError) as e:        # no loading
        cap.getCaponGPU(x, 0.0, 16, 1, form=F, loading=A)
    assert e.value.status == _lib.ERR_LAUNCH
    with pytest.raises(_lib.CaponError) as e:        # negative segment
        cap.getCaponGPU(x, 0.5, 16, 1, form=F, loading=A, segment=-1)
    assert e.value.status == _lib.ERR_LAUNCH
