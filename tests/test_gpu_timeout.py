"""The device-timeout status path, exercised without a GPU fault.

Every wait inside the fused kernel is bounded.  With COS_CAPON_TEST_STALL=1
each CTA waits on a shared-memory barrier that nothing completes, so the
bounded wait gives up: the kernel records the timeout in the context's status
word, lets its own bulk copies land, and returns.  The call must report
COS_CAPON_ERR_TIMEOUT (909, cudaErrorTimeout), and the context must stay
usable: the next call succeeds and reproduces the earlier outputs bit for bit.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cube(Nx, Ny, M, seed=11):
    rng = np.random.default_rng(seed)
    return ((rng.standard_normal((Nx, Ny, M)) + 1j * rng.standard_normal((Nx, Ny, M))) / np.sqrt(2)).astype(
        np.complex64)


@pytest.mark.parametrize("want_w", [False, True])
def test_stalled_wait_reports_timeout_and_context_recovers(want_w):
    from cos_gb300 import _lib, capon
    Nx, Ny, M, L, K = 24, 300, 32, 16, 1
    npy = Ny - 2 * K
    x = _cube(Nx, Ny, M)
    ctx = capon.Capon()

    def call():
        z = np.zeros((Nx, npy), np.complex64)
        P = np.zeros((Nx, npy), np.float32)
        w = np.zeros((Nx, npy, L), np.complex64) if want_w else None
        rc = ctx.getCaponEx(z, P, w, None, x, 0.01, L, K, M, Nx, Ny, 0, capon.opts())
        return rc, z, P, w

    rc, z0, P0, w0 = call()            # first call of the shape also runs the autotuner
    assert rc == 0
    os.environ["COS_CAPON_TEST_STALL"] = "1"
    try:
        rc, _, _, _ = call()
    finally:
        del os.environ["COS_CAPON_TEST_STALL"]
    assert rc == _lib.ERR_TIMEOUT == 909
    assert ctx.device_status() == 0    # the status word was cleared when the timeout was reported
    rc, z1, P1, w1 = call()
    assert rc == 0
    np.testing.assert_array_equal(z1, z0)
    np.testing.assert_array_equal(P1, P0)
    if want_w:
        np.testing.assert_array_equal(w1, w0)
