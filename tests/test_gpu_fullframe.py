"""Full-frame parity: every pixel of whole configuration frames, not slices.

* Config 0 ([Nx=128][Ny=512][M=32], L=16, K=1), the reference's own CPU-sized
  case, through the drop-in entry points (getCaponCUDAPy -> Capon::getCapon,
  and getCaponGPU with the output power) against the FP64 oracle on every
  pixel, and -- where the reference's own CPU path is built
  (getCaponC.getCaponCPy, getCaponC.pyx:61-94) -- the oracle against the
  reference on every pixel: z and w directly, zPow (the reference's
  upper-triangle power, getCaponC.pyx:285-289) exactly as it computes it.
* Config 1 ([256][2048][64], L=32, K=2: 523,264 pixels) through the device
  API, the FP32 fused form and the tensor-core fused form, against the
  threaded FP64 oracle on every pixel.

Errors are printed as max and median; the bars are the fused form's.
"""
import os

import numpy as np
import pytest

import oracle
import ref

pytestmark = pytest.mark.gpu

TOL_P = 1e-4
TOL_Z = 1e-3
TOL_W = 2e-3


def _report(what, e):
    print(f"{what}: " + ", ".join(f"{k} max {v.max():.2e} med {np.median(v):.2e}" for k, v in e.items()))


def test_config0_full_frame():
    from cos_gb300 import capon, synth
    c = synth.config0(seed=0)
    x, d, L, K = c["x"], c["d"], c["L"], c["K"]
    o = oracle.capon(x, d, L, K, nthreads=os.cpu_count() or 1)
    z, R, w, e = capon.getCaponCUDAPy(x, d, L, K, np.array([0]), False, False, want_R=False)
    assert e == 0
    z2, P2, w2 = capon.getCaponGPU(x, d, L, K)
    err = {"P": np.abs(P2 - o["P"]) / o["P"],
           "z": np.abs(z - o["z"]) / np.sqrt(o["P"]),
           "w": np.linalg.norm(w - o["w"], axis=-1) / np.linalg.norm(o["w"], axis=-1)}
    _report(f"config0 full frame ({x.shape[0] * (x.shape[1] - 2 * K)} pixels) vs FP64 oracle", err)
    assert err["P"].max() <= TOL_P and err["z"].max() <= TOL_Z and err["w"].max() <= TOL_W
    # the two drop-in calls run the same kernels on the same frame
    assert np.array_equal(z, z2) and np.array_equal(w, w2)
    if not ref.available():
        pytest.skip("reference CPU path not built here; GPU checked against the oracle only")
    r = ref.load().getCaponCPy(x.astype(np.complex128), d, L, K, np.array([]), False, False)
    zr, zpow_r, wr = (np.asarray(a) for a in r)
    scale = np.sqrt(o["P"])
    eo = {"z": np.abs(o["z"] - zr) / scale, "zPow": np.abs(o["zpow"] - zpow_r) / np.abs(zpow_r),
          "w": np.linalg.norm(o["w"] - wr, axis=-1) / np.linalg.norm(wr, axis=-1)}
    _report("config0 full frame: oracle vs reference getCaponCPy", eo)
    assert eo["z"].max() <= 1e-10 and eo["zPow"].max() <= 1e-10 and eo["w"].max() <= 1e-10
    eg = {"z": np.abs(z - zr) / scale,
          "w": np.linalg.norm(w - wr, axis=-1) / np.linalg.norm(wr, axis=-1)}
    _report("config0 full frame: GPU drop-in vs reference getCaponCPy", eg)
    assert eg["z"].max() <= TOL_Z and eg["w"].max() <= TOL_W


@pytest.mark.parametrize("form", [0, 6])
def test_config1_full_frame(form):
    import torch
    from cos_gb300 import capon, synth
    c = synth.config1(seed=1)
    x, d, L, K = c["x"], c["d"], c["L"], c["K"]
    Nx, Ny, _ = x.shape
    f = capon.DeviceFrame(x=torch.from_numpy(x).cuda(), L=L, K=K, d=d)
    f.P = torch.empty((Nx, Ny - 2 * K), dtype=torch.float32, device="cuda")
    capon.capon_frames([f], o=capon.opts(form=form))
    torch.cuda.synchronize()
    z, P = f.z.cpu().numpy(), f.P.cpu().numpy()
    o = oracle.capon(x, d, L, K, want_w=False, nthreads=os.cpu_count() or 1)
    err = {"P": np.abs(P - o["P"]) / o["P"], "z": np.abs(z - o["z"]) / np.sqrt(o["P"])}
    _report(f"config1 full frame form {form} ({Nx * (Ny - 2 * K)} pixels) vs FP64 oracle", err)
    assert np.all(np.isfinite(P)) and np.all(np.isfinite(z))
    assert err["P"].max() <= TOL_P and err["z"].max() <= TOL_Z
