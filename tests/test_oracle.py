"""The FP64 oracle pinned against the reference: its linear-algebra known
answers (framework/linalg/tests) and outputs of the reference's own CPU Capon
path (getCaponC.getCaponCPy) on seeded inputs.  CPU only."""
import os

import numpy as np
import pytest

import oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")
KA = np.load(os.path.join(GOLD, "linalg_known_answers.npz"))
CASES = np.load(os.path.join(GOLD, "capon_ref_cases.npz"))


def test_cholesky_known_answers():
    # testCholesky.py:16-23 (real tridiagonal) and :61-68 (complex Hermitian), 14 places
    np.testing.assert_allclose(oracle.cholesky(KA["A"]), KA["R"], atol=1e-14)
    np.testing.assert_allclose(oracle.cholesky(KA["complexA"]), KA["complexR"], atol=1e-14)
    U = oracle.cholesky(KA["complexA"])
    np.testing.assert_allclose(U.conj().T @ U, KA["complexA"], atol=1e-13)


def test_triangular_solves_known_answers():
    # testCholesky.py:40-58 and :70-82; testLinearSolvec.py:145-154
    U = oracle.cholesky(KA["A"])
    for b, x in (("b1", "x1"), ("b2", "x2")):
        y = oracle.forward_solve(U.conj().T, KA[b])
        np.testing.assert_allclose(oracle.back_solve(U, y), KA[x], atol=1e-14)
    U = oracle.cholesky(KA["complexA"])
    y = oracle.forward_solve(U.conj().T, KA["complexb"])
    np.testing.assert_allclose(y, KA["complexy"], atol=1e-14)
    np.testing.assert_allclose(oracle.back_solve(U, y), KA["complexx"], atol=1e-14)
    np.testing.assert_array_equal(oracle.back_solve(KA["C"], KA["b1c"]), KA["x1c"])
    np.testing.assert_array_equal(oracle.forward_solve(KA["C"].conj().T, KA["b1c"]), KA["x1cT"])


def test_solve_cholesky_known_answers():
    # testLinearSolvec.py:119-129
    np.testing.assert_allclose(oracle.solve_cholesky(KA["A"], KA["b1"]), KA["x1"], atol=1e-14)
    np.testing.assert_allclose(oracle.solve_cholesky(KA["complexA"], KA["complexb"]), KA["complexx"], atol=1e-14)
    rng = np.random.default_rng(5)
    L = 24
    U = np.triu(rng.standard_normal((L, L)) + 1j * rng.standard_normal((L, L))) + np.eye(L) * 100
    A = U.conj().T @ U
    b = rng.standard_normal(L) + 1j * rng.standard_normal(L)
    np.testing.assert_allclose(oracle.solve_cholesky(A, b), np.linalg.solve(A, b), rtol=1e-12, atol=1e-15)


def test_butler_known_answers():
    # testBeamspace.py:14-29 (first-Nb-bins layout of beamspace.butlerMatrix)
    np.testing.assert_allclose(oracle.butler(4, 4, symmetric=False), KA["but4"], atol=1e-15)
    np.testing.assert_allclose(oracle.butler(3, 3, symmetric=False), KA["but3"], atol=1e-15)
    np.testing.assert_allclose(oracle.butler(2, 3, symmetric=False) @ KA["complexb"], KA["bsComplexb"], atol=1e-14)
    # the GPU layout agrees with it whenever Nb is odd or Nb < L ... for these sizes
    np.testing.assert_allclose(oracle.butler(3, 3), KA["but3"], atol=1e-15)
    np.testing.assert_allclose(oracle.butler(2, 3) @ KA["complexb"], KA["bsComplexb"], atol=1e-14)


def test_butler_gpu_layout_bins():
    # capon_kernel.cu:53-59: beams above Nb/2 take the negative bins
    B = oracle.butler(5, 64)
    bins = np.round(np.angle(B[:, 1]) / (-2 * np.pi / 64)).astype(int) % 64
    assert list(bins) == [0, 1, 2, 62, 63]
    np.testing.assert_allclose(B @ B.conj().T, np.eye(5), atol=1e-14)


@pytest.mark.parametrize("i", range(len(CASES["cases"])))
def test_oracle_matches_reference_cpu_path(i):
    Nx, Ny, M, L, K, d, _seed = CASES["cases"][i]
    x = CASES[f"x{i}"]
    o = oracle.capon(x, d, int(L), int(K))
    zr, zpr, wr = CASES[f"z{i}"], CASES[f"zpow{i}"], CASES[f"w{i}"]
    assert o["z"].shape == zr.shape and o["w"].shape == wr.shape
    np.testing.assert_allclose(o["z"], zr, rtol=1e-10, atol=1e-12 * np.abs(zr).max())
    np.testing.assert_allclose(o["zpow"], zpr, rtol=1e-10, atol=1e-12 * np.abs(zpr).max())
    np.testing.assert_allclose(o["w"], wr, rtol=1e-9, atol=1e-11 * np.abs(wr).max())


def test_power_definitions():
    """P = w^H R_d w = 1/Re(a^H R_d^-1 a); the reference's zPow satisfies
    2 Re(zPow) - sum_i R_ii |w_i|^2 = w^H conj(R_d) w (upper-triangle sum of
    w_i R_ij conj(w_j))."""
    i = 0
    Nx, Ny, M, L, K, d, _ = CASES["cases"][i]
    o = oracle.capon(CASES[f"x{i}"], d, int(L), int(K), want_R=True)
    R, w = o["R"], o["w"]
    np.testing.assert_allclose(np.einsum("xyi,xyij,xyj->xy", w.conj(), R, w).real, o["P"], rtol=1e-12)
    lhs = 2 * CASES[f"zpow{i}"].real - np.einsum("xyii,xyi->xy", R, np.abs(w) ** 2).real
    rhs = np.einsum("xyi,xyij,xyj->xy", w.conj(), R.conj(), w).real
    np.testing.assert_allclose(lhs, rhs, rtol=1e-10)


def test_oracle_threads_identical():
    x = CASES["x0"]
    a = oracle.capon(x, 0.01, 16, 1, nthreads=1)
    b = oracle.capon(x, 0.01, 16, 1, nthreads=3)
    for k in ("z", "zpow", "P", "w"):
        np.testing.assert_array_equal(a[k], b[k])


def test_beamspace_full_dft_equals_element_space():
    # with Nb = L (odd) the Butler matrix is unitary, so beamspace Capon with
    # either loading convention reproduces element-space Capon exactly
    rng = np.random.default_rng(7)
    x = (rng.standard_normal((2, 14, 12)) + 1j * rng.standard_normal((2, 14, 12))).astype(np.complex64)
    e = oracle.capon(x, 0.05, 5, 1)
    for bsl in (False, True):
        b = oracle.capon(x, 0.05, 5, 1, Nb=5, bs_loading=bsl)
        np.testing.assert_allclose(b["z"], e["z"], rtol=1e-9, atol=1e-12)
        np.testing.assert_allclose(b["P"], e["P"], rtol=1e-9)
        np.testing.assert_allclose(b["w"], e["w"], rtol=1e-9, atol=1e-12)


def test_beamspace_reduces_dimension():
    rng = np.random.default_rng(8)
    x = (rng.standard_normal((2, 12, 16)) + 1j * rng.standard_normal((2, 12, 16))).astype(np.complex64)
    b = oracle.capon(x, 0.01, 8, 1, Nb=3)
    # w lies in the span of the Butler rows: w = B^H w_bs
    B = oracle.butler(3, 8)
    w = b["w"].reshape(-1, 8)
    proj = w @ B.conj().T @ B
    np.testing.assert_allclose(proj, w, atol=1e-12)
    assert np.all(b["P"] > 0)


@pytest.mark.parametrize("bad", [
    dict(L=0), dict(L=20), dict(K=-1), dict(K=6), dict(Nb=9), dict(Nb=-1),
])
def test_oracle_rejects_invalid_sizes(bad):
    args = dict(L=8, K=1, Nb=0)
    args.update(bad)
    x = np.zeros((2, 12, 16), np.complex64)
    with pytest.raises(ValueError):
        oracle.capon(x, 0.01, args["L"], args["K"], Nb=args["Nb"])


def test_reference_cpu_path_live():
    """When the reference's compiled CPU path is present, re-run it on a fresh
    seeded case (beyond the committed fixtures)."""
    import ref
    if not ref.available():
        pytest.skip("reference CPU path not built here")
    g = ref.load()
    rng = np.random.default_rng(99)
    x = (rng.standard_normal((2, 22, 20)) + 1j * rng.standard_normal((2, 22, 20))).astype(np.complex64)
    zr, zpr, wr = g.getCaponCPy(x.astype(np.complex128), 0.02, 7, 2, np.array([]), False, False)
    o = oracle.capon(x, 0.02, 7, 2)
    np.testing.assert_allclose(o["z"], zr, rtol=1e-10, atol=1e-13)
    np.testing.assert_allclose(o["w"], wr, rtol=1e-9, atol=1e-12)


def _numpy_capon_fb(x, regCoef, L, K, fb):
    """Per-pixel restatement of getCaponPy_ref.py:86-121 (R from the snapshot
    matrix d, optional R = (R + J R^T J)/2, loading regCoef*tr(R)/L, w, z, P)."""
    Nx, Ny, M = x.shape
    Ns, T = M - L + 1, 2 * K + 1
    J = np.fliplr(np.eye(L))
    out = np.zeros((Nx, Ny - 2 * K)), np.zeros((Nx, Ny - 2 * K), complex)
    for b in range(Nx):
        for p in range(Ny - 2 * K):
            d = np.array([x[b, p + t, s:s + L] for t in range(T) for s in range(Ns)]).astype(complex)
            R = d.T @ d.conj() / (Ns * T)          # R[j,k] = sum x[s+j] conj(x[s+k])
            if fb:
                R = 0.5 * (R + J @ R.T @ J)
            g = x[b, p + K].astype(complex)
            g = np.array([g[l:l + Ns].sum() for l in range(L)]) / Ns
            Rd = R + regCoef * np.trace(R) / L * np.eye(L)
            Ria = np.linalg.solve(Rd, np.ones(L))
            w = Ria / Ria.sum()
            out[0][b, p] = 1.0 / Ria.sum().real
            out[1][b, p] = np.vdot(w, g)
    return out


@pytest.mark.parametrize("fb", [False, True])
def test_forward_backward_averaging_matches_numpy_restatement(fb):
    rng = np.random.default_rng(11)
    x = (rng.standard_normal((2, 10, 12)) + 1j * rng.standard_normal((2, 10, 12))).astype(np.complex64)
    x[:, :, :] += 4.0 * np.exp(1j * 0.9 * np.arange(12))
    P, z = _numpy_capon_fb(x, 0.05, 5, 1, fb)
    o = oracle.capon(x, 0.05, 5, 1, fb=fb, fp32_scalars=False)
    np.testing.assert_allclose(o["P"], P, rtol=1e-10)
    np.testing.assert_allclose(o["z"], z, rtol=1e-9, atol=1e-12)
    if fb:  # the averaging changes the answer on this (non-persymmetric) data
        o0 = oracle.capon(x, 0.05, 5, 1, fp32_scalars=False)
        assert np.abs(o0["P"] - o["P"]).max() > 1e-6 * np.abs(o["P"]).max()


def test_forward_backward_equals_flipped_conjugate_rows():
    """(R + J R^T J)/2 is the mean of the covariances of x and of
    x~[m] = conj(x[M-1-m]) -- the identity the beamspace kernel uses."""
    rng = np.random.default_rng(12)
    x = (rng.standard_normal((2, 9, 14)) + 1j * rng.standard_normal((2, 9, 14))).astype(np.complex64)
    L, K = 6, 1
    a = oracle.capon(x, 0.0, L, K, want_R=True, fb=True, fp32_scalars=False)["R"]
    xt = np.ascontiguousarray(np.conj(x[:, :, ::-1]))
    r0 = oracle.capon(x, 0.0, L, K, want_R=True, fp32_scalars=False)["R"]
    r1 = oracle.capon(xt, 0.0, L, K, want_R=True, fp32_scalars=False)["R"]
    np.testing.assert_allclose(a, 0.5 * (r0 + r1), rtol=1e-12, atol=1e-12)


def test_general_subspace_matches_numpy_restatement():
    """Beamspace over a caller-given V against a per-pixel restatement of
    getCaponAllC.pyx:226-231, 346-440 (element loading before the transform,
    a = V 1, R = V R_d V^H, g_bs = V g, w_bs = R^-1 a / a^H R^-1 a,
    z = w_bs^H g_bs); the oracle reports w = V^H w_bs-normalised weights."""
    rng = np.random.default_rng(13)
    M, L, K, Nb = 14, 8, 1, 3
    x = (rng.standard_normal((2, 9, M)) + 1j * rng.standard_normal((2, 9, M))).astype(np.complex64)
    x += (3.0 * np.exp(1j * 0.7 * np.arange(M))).astype(np.complex64)
    V = rng.standard_normal((Nb, L)) + 1j * rng.standard_normal((Nb, L))
    for bs_loading in (False, True):
        o = oracle.capon(x, 0.05, L, K, Nb=Nb, V=V, bs_loading=bs_loading, fp32_scalars=False)
        Ns, T = M - L + 1, 2 * K + 1
        for b in range(2):
            for p in range(9 - 2 * K):
                d = np.array([x[b, p + t, s:s + L] for t in range(T) for s in range(Ns)]).astype(complex)
                R = d.T @ d.conj() / (Ns * T)
                g = np.array([x[b, p + K, l:l + Ns].astype(complex).sum() for l in range(L)]) / Ns
                if not bs_loading:
                    R = R + 0.05 * np.trace(R) / L * np.eye(L)
                Rb = V @ R @ V.conj().T
                if bs_loading:
                    Rb = Rb + 0.05 * np.trace(Rb) / Nb * np.eye(Nb)
                a = V @ np.ones(L)
                Ria = np.linalg.solve(Rb, a)
                aRia = np.vdot(a, Ria)
                wb = Ria / aRia
                np.testing.assert_allclose(o["z"][b, p], np.vdot(wb, V @ g), rtol=1e-9)
                np.testing.assert_allclose(o["P"][b, p], 1.0 / aRia.real, rtol=1e-9)


WOOD = np.load(os.path.join(GOLD, "woodbury_ref_cases.npz"))


@pytest.mark.parametrize("i", range(len(WOOD["cases"])))
def test_sherman_morrison_matches_reference_woodbury(i):
    # iterativeBuildUpRinv / iterativeBuildDownRinv (woodburyc.pyx:15-42) outputs
    M, L, n, _ = (int(v) for v in WOOD["cases"][i])
    B, X = WOOD[f"B0_{i}"], WOOD[f"X_{i}"]
    for r in range(n):
        B, den = oracle.sm_row(B, X[r], L, +1)
        assert den > 1.0
        np.testing.assert_allclose(B, WOOD[f"up_{i}"][r], rtol=0, atol=1e-13 * np.abs(B).max())
    Bd, _ = oracle.sm_row(B, X[0], L, -1)
    np.testing.assert_allclose(Bd, WOOD[f"down_{i}"], rtol=0, atol=1e-12 * np.abs(Bd).max())


def test_sliding_inverse_matches_reference_woodbury_driver():
    # the sliding-window Capon case computed with the reference's own update functions
    Nx, Ny, M, L, K, d, seg, _ = WOOD["slide_params"]
    o = oracle.capon_sliding(WOOD["slide_x"], float(d), int(L), int(K), int(seg))
    np.testing.assert_allclose(o["P"], WOOD["slide_P"], rtol=1e-12)
    np.testing.assert_allclose(o["w"], WOOD["slide_w"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(o["z"], WOOD["slide_z"], rtol=0, atol=1e-12 * np.abs(WOOD["slide_z"]).max())


@pytest.mark.parametrize("seg", [1, 6, 10_000])
def test_sliding_inverse_equals_direct_solve(seg):
    # in FP64 the tracked inverse and a Cholesky solve per pixel agree
    # (absolute loading), whatever the segment length
    rng = np.random.default_rng(31)
    x = (rng.standard_normal((3, 60, 32)) + 1j * rng.standard_normal((3, 60, 32))).astype(np.complex64)
    x += (5.0 * np.exp(1j * 0.4 * np.arange(32))[None, None, :]).astype(np.complex64)
    a = oracle.capon_sliding(x, 0.2, 16, 1, seg)
    b = oracle.capon(x, 0.2, 16, 1, absolute=True, fp32_scalars=False)
    np.testing.assert_allclose(a["P"], b["P"], rtol=1e-10)
    np.testing.assert_allclose(a["w"], b["w"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(a["z"], b["z"], rtol=0, atol=1e-10 * np.abs(b["z"]).max())
    assert a["den_min"] > 0.0


def test_sliding_inverse_rejects_invalid():
    x = np.zeros((1, 10, 8), np.complex64)
    for args in ((0.2, 4, 1, 0), (0.0, 4, 1, 3), (0.2, 9, 1, 3), (0.2, 4, 5, 3)):
        with pytest.raises(ValueError):
            oracle.capon_sliding(x, *args)


# ---- getCaponAllC (the reference's all-options CPU Capon), pinned to runs of
# the reference itself: tests/golden/capon_all_ref_cases.npz

def _all_gold():
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "capon_all_ref_cases.npz"))


def test_forward_backward_matches_reference_getCaponAllC():
    """doFBAvg (getCaponAllC.pyx:346-347) with its default Cholesky solver:
    the oracle's forward-backward averaged covariance gives the reference's z,
    zPow and w.  The reference averages only the upper triangle it built; the
    upper triangle of (R + J R^T J)/2 depends only on R's upper triangle, so
    the two agree exactly."""
    g = _all_gold()
    for i, (Nx, Ny, M, L, K, d, _s) in enumerate(g["fb_cases"]):
        x = g[f"fb_x{i}"]
        o = oracle.capon(x, d, int(L), int(K), fb=True)
        zr = g[f"fb_z{i}"]
        np.testing.assert_allclose(o["z"], zr, rtol=0, atol=1e-11 * np.abs(zr).max())
        np.testing.assert_allclose(o["zpow"], g[f"fb_zpow{i}"], rtol=1e-10)
        np.testing.assert_allclose(o["w"], g[f"fb_w{i}"], rtol=0, atol=1e-11 * np.abs(g[f"fb_w{i}"]).max())


@pytest.mark.parametrize("tag,bs_loading", [("full_bsload", True), ("full_elload", False)])
def test_general_subspace_matches_reference_getCaponAllC(tag, bs_loading):
    """A general V (BEAMSPACE, getCaponAllC.pyx:365-386) through the branch
    that restores R's lower triangle before R_bs = V R V^H, loading after the
    transform with tr(R_bs)/Nb (DIAGONAL_LOADING_IN_BEAMSPACE) or before it
    with tr(R)/L: the oracle's z and its element-space weights V^H w_bs equal
    the reference's."""
    g = _all_gold()
    Nx, Ny, M, L, K, d, Nb, _s = g["v_case"]
    L, K, Nb = int(L), int(K), int(Nb)
    x, V = g["v_x"], g["v_V"]
    o = oracle.capon(x, d, L, K, Nb=Nb, V=V, bs_loading=bs_loading)
    zr, wbs = g[f"v_{tag}_z"], g[f"v_{tag}_w"]
    np.testing.assert_allclose(o["z"], zr, rtol=0, atol=1e-11 * np.abs(zr).max())
    wel = np.einsum("bl,xyb->xyl", V.conj(), wbs)
    np.testing.assert_allclose(o["w"], wel, rtol=0, atol=1e-10 * np.abs(wel).max())


def test_reference_default_subspace_branch_uses_a_half_filled_R():
    """The reference's default solver with a general V transforms the
    covariance it built as an upper triangle only (its lower triangle is
    restored only for the numpy solver, getCaponAllC.pyx:320-326), so
    R_bs = V R_upper V^H is not Hermitian.  This restates exactly that -- the
    upper triangle of the normalised R, the transform, loading tr(R_bs)/Nb,
    the Cholesky with complex pivots that reads R_bs's upper triangle -- and
    matches the
    reference; the oracle and the GPU path use the full R instead, and differ
    from this branch by far more than rounding."""
    g = _all_gold()
    Nx, Ny, M, L, K, d, Nb, _s = g["v_case"]
    M, L, K, Nb = int(M), int(L), int(K), int(Nb)
    x, V = g["v_x"].astype(np.complex128), g["v_V"]
    Ns, T = M - L + 1, 2 * K + 1
    zr = g["v_upper_bsload_z"]
    z = np.zeros_like(zr)
    for bx in range(x.shape[0]):
        for p in range(x.shape[1] - 2 * K):
            X = x[bx, p:p + T]
            Rf = X.T.conj() @ X                                   # R_full[i,j] = sum_t conj(x_i) x_j
            R = sum(Rf[s:s + L, s:s + L] for s in range(Ns))
            # the upper triangle it keeps, conj * norm_inv (an FP32 scalar there, as K_inv)
            Ru = np.triu(R.conj()) * float(np.float32(1.0 / (Ns * T)))
            Rbs = V @ Ru @ V.conj().T
            Rbs += np.trace(Rbs) * np.float32(d) / Nb * np.eye(Nb)
            # its Cholesky reads the upper triangle and takes complex square
            # roots of the (here complex) pivots (matrixDecompc.pyx:19-50),
            # then U^H y = a, U x = y (linearSolvec.pyx:312-346)
            U = np.zeros((Nb, Nb), complex)
            for i in range(Nb):
                U[i, i] = np.sqrt(Rbs[i, i] - np.sum(U[:i, i].conj() * U[:i, i]))
                for j in range(i + 1, Nb):
                    U[i, j] = (Rbs[i, j] - np.sum(U[:i, i].conj() * U[:i, j])) / U[i, i]
            a = V @ np.ones(L)
            y = np.zeros(Nb, complex)
            for i in range(Nb):
                y[i] = (a[i] - np.sum(U[:i, i].conj() * y[:i])) / U[i, i].conj()
            ria = np.zeros(Nb, complex)
            for i in reversed(range(Nb)):
                ria[i] = (y[i] - np.sum(U[i, i + 1:] * ria[i + 1:])) / U[i, i]
            w = ria / (a.conj() @ ria)
            gs = V @ np.array([x[bx, p + K, i:i + Ns].sum() * float(np.float32(1.0 / Ns)) for i in range(L)])
            z[bx, p] = np.sum(w.conj() * gs)
    np.testing.assert_allclose(z, zr, rtol=0, atol=1e-11 * np.abs(zr).max())
    o = oracle.capon(g["v_x"], d, L, K, Nb=Nb, V=V, bs_loading=True)
    assert np.max(np.abs(o["z"] - zr)) > 1e-3 * np.abs(zr).max()


def test_fp32_factorisation_limit_on_the_precision_stress_case():
    """What FP32 arithmetic can reach on the config-3 stress data (two coherent
    scatterers one beam apart at 40 dB, loading 1e-3, L=64, K=4), with the
    oracle's FP64 R as input: rounded once to complex64 and factored by
    single-precision LAPACK, the output power misses 1e-4 on the most
    ill-conditioned pixels (cond ~3e4); one refinement step with an FP64
    residual against the exact R brings every pixel within 1e-6.  The GPU
    kernels' bars for this data (tests/test_gpu_wide.py) follow from it."""
    import scipy.linalg as sl
    from cos_gb300 import synth
    x = synth.cube(200, 3, 128, [100.0, 100.0], seed=3, coherent_pair=True)
    x = np.ascontiguousarray(x[2:, 60:120])   # the pair's beam, the scatterers' range
    o = oracle.capon(x, 1e-3, 64, 4, want_w=False, want_R=True, nthreads=os.cpu_count() or 1)
    a = np.ones(64)
    e0, e1 = [], []
    for R, P in zip(o["R"].reshape(-1, 64, 64), o["P"].ravel()):
        c = sl.cho_factor(R.astype(np.complex64))
        x0 = sl.cho_solve(c, a.astype(np.complex64)).astype(np.complex128)
        x1 = x0 + sl.cho_solve(c, (a - R @ x0).astype(np.complex64))
        e0.append(abs(1 / np.real(a @ x0) - P) / P)
        e1.append(abs(1 / np.real(a @ x1) - P) / P)
    assert max(e0) > 1e-4
    assert max(e1) < 1e-6
