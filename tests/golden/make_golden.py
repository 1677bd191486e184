"""Generate the golden fixtures under tests/golden/ from the reference itself.

Run where the reference sources and its compiled CPU path exist
(``python oracle/build_ref.py`` first):

    python tests/golden/make_golden.py

Writes
* ``linalg_known_answers.npz`` -- the known-answer arrays of the reference's
  linear-algebra tests, read (not retyped) from
  framework/linalg/tests/testMatrixOperations.py:12-90 by parsing its
  ``setUp`` with ``ast``: the 3x3 real and complex Hermitian matrices with
  their Cholesky factors, right-hand sides and solutions, the 3x3 / 4x4
  Butler matrices and the 2x3 beamspace transform of ``complexb``.
* ``woodbury_ref_cases.npz`` -- rank-1 updates and downdates of an inverse by
  the reference's framework/linalg/woodburyc.pyx (iterativeBuildUpRinv /
  iterativeBuildDownRinv) on seeded rows, and a small sliding-window Capon
  case driven by those two functions (the reference's own build-up,
  iterativeBuildRinv, seeds with a real-typed identity that its complex
  buffer declaration rejects, so the build-up here starts from a complex one).
* ``capon_ref_cases.npz`` -- seeded inputs and the outputs of the
  reference's own getCaponC.getCaponCPy (z, zPow, w; complex128) for small
  cases covering K = 0, L = 1, L = M, one valid range row, and the
  (M, L, K) of the benchmark configurations.
* ``capon_all_ref_cases.npz`` -- outputs of the reference's
  getCaponAllC.getCaponCPy: forward-backward averaging in element space, and
  a general subspace V through the branch that restores R's lower triangle
  (both loading orders) and through its default solver.
* ``lca_ref_cases.npz`` -- outputs of the reference's lcac.lca and lcacx.lca
  for 1 x 1, all-ones column, general and weighted filters.
* ``tdib_ref_cases.npz`` -- outputs of the reference's tdibC.tdib on seeded
  steering geometries (some pixels beyond the time axis).
"""
from __future__ import annotations

import ast
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
# the reference tree: $COS_REFERENCE_ROOT, else a checkout beside this repository
REF = os.environ.get("COS_REFERENCE_ROOT", os.path.join(ROOT, "..", "reference"))
sys.path.insert(0, ROOT)

# attribute name in setUp -> fixture key
KNOWN = ["A", "R", "b1", "x1", "b2", "x2", "C", "b1c", "x1c", "x1cT", "complexA", "complexR", "complexb",
         "complexy", "complexx", "but4", "but3", "bsComplexb"]

# (Nx, Ny, M, L, K, regCoef, seed)
CASES = [
    (3, 40, 32, 16, 1, 0.01, 10),    # config-0 (M, L, K)
    (2, 24, 64, 32, 2, 0.01, 11),    # config-1 (M, L, K)
    (2, 20, 12, 6, 0, 0.2, 12),      # K = 0
    (2, 12, 10, 3, 1, 0.01, 13),     # odd M, small L
    (2, 10, 8, 8, 1, 0.05, 14),      # L = M (one subarray)
    (2, 9, 5, 1, 4, 0.01, 15),       # L = 1 and Ny = 2K+1 (one pixel row)
    (2, 16, 96, 48, 1, 0.01, 16),    # config-2 frame 3 element-space size
]


def _num(node):
    """Evaluate a numeric expression tree: numbers, lists, +, -, *, / only."""
    if isinstance(node, ast.Constant) and isinstance(node.value, (int, float, complex)):
        return node.value
    if isinstance(node, ast.List):
        return [_num(e) for e in node.elts]
    if isinstance(node, ast.UnaryOp) and isinstance(node.op, (ast.USub, ast.UAdd)):
        v = _num(node.operand)
        return -v if isinstance(node.op, ast.USub) else v
    if isinstance(node, ast.BinOp) and isinstance(node.op, (ast.Add, ast.Sub, ast.Mult, ast.Div)):
        a, b = _num(node.left), _num(node.right)
        if isinstance(node.op, ast.Add):
            return a + b
        if isinstance(node.op, ast.Sub):
            return a - b
        if isinstance(node.op, ast.Mult):
            return a * b  # also list repetition, e.g. [0.5]*4
        return a / b
    raise ValueError(f"unsupported expression: {ast.dump(node)}")


def _literal(node):
    """Value of np.array([...], dtype=complex) in setUp, else None."""
    if isinstance(node, ast.Call) and getattr(node.func, "attr", "") == "array":
        return np.array(_num(node.args[0]), dtype=complex)
    return None


def known_answers() -> dict:
    path = os.path.join(REF, "framework/linalg/tests/testMatrixOperations.py")
    tree = ast.parse(open(path).read())
    out = {}
    for node in ast.walk(tree):
        if isinstance(node, ast.FunctionDef) and node.name == "setUp":
            for st in node.body:
                if isinstance(st, ast.Assign) and isinstance(st.targets[0], ast.Attribute):
                    name = st.targets[0].attr
                    if name in KNOWN:
                        v = _literal(st.value)
                        if v is not None:
                            out[name] = v
    missing = [k for k in KNOWN if k not in out]
    if missing:
        raise RuntimeError(f"known answers not found: {missing}")
    return out


def ref_cases() -> dict:
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref  # noqa: E402
    g = ref.load()
    out = {"cases": np.array(CASES, dtype=np.float64)}
    for i, (Nx, Ny, M, L, K, d, seed) in enumerate(CASES):
        rng = np.random.default_rng(seed)
        x = (rng.standard_normal((Nx, Ny, M)) + 1j * rng.standard_normal((Nx, Ny, M))).astype(np.complex64)
        # a coherent plane wave on top of the noise, so R is not close to white
        m = np.arange(M)
        x += (4.0 * np.exp(1j * 0.7 * m)[None, None, :]).astype(np.complex64)
        z, zpow, w = g.getCaponCPy(x.astype(np.complex128), float(d), int(L), int(K), np.array([]), False, False)
        out[f"x{i}"] = x
        out[f"z{i}"] = z
        out[f"zpow{i}"] = zpow
        out[f"w{i}"] = w
    return out


# (M, L, rows, seed) for the update / downdate cases
WOOD_CASES = [(8, 4, 3, 20), (12, 6, 4, 21), (10, 10, 3, 22), (64, 32, 2, 23)]
# sliding-window case: (Nx, Ny, M, L, K, d, segment, seed)
WOOD_SLIDE = (2, 20, 12, 6, 1, 0.3, 5, 24)


def woodbury_cases() -> dict:
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref  # noqa: E402
    ref._prepare()
    from framework.linalg import woodburyc as wb  # noqa: E402
    out = {"cases": np.array(WOOD_CASES, dtype=np.int64)}
    for i, (M, L, n, seed) in enumerate(WOOD_CASES):
        rng = np.random.default_rng(seed)
        G = rng.standard_normal((L, 2 * L)) + 1j * rng.standard_normal((L, 2 * L))
        B0 = np.linalg.inv(G @ G.conj().T / (2 * L) + 0.5 * np.eye(L))
        X = rng.standard_normal((n, M)) + 1j * rng.standard_normal((n, M))
        B = B0.copy()
        ups = []
        for r in range(n):
            B = wb.iterativeBuildUpRinv(B, X[r], M, L)
            ups.append(B)
        down = wb.iterativeBuildDownRinv(B, X[0], M, L)
        out[f"B0_{i}"], out[f"X_{i}"] = B0, X
        out[f"up_{i}"], out[f"down_{i}"] = np.array(ups), down
    # sliding-window Capon driven by the reference's update functions
    Nx, Ny, M, L, K, d, seg, seed = WOOD_SLIDE
    rng = np.random.default_rng(seed)
    x = (rng.standard_normal((Nx, Ny, M)) + 1j * rng.standard_normal((Nx, Ny, M))).astype(np.complex64)
    x += (3.0 * np.exp(1j * 0.9 * np.arange(M))[None, None, :]).astype(np.complex64)
    T, Ns, npy = 2 * K + 1, M - L + 1, Ny - 2 * K
    xd = x.astype(np.complex128)
    z = np.zeros((Nx, npy), complex)
    P = np.zeros((Nx, npy))
    w = np.zeros((Nx, npy, L), complex)
    for bx in range(Nx):
        for p0 in range(0, npy, seg):
            B = np.eye(L, dtype=complex) / (Ns * T * d)
            for t in range(p0, p0 + T):
                B = wb.iterativeBuildUpRinv(B, xd[bx, t], M, L)
            for p in range(p0, min(p0 + seg, npy)):
                if p > p0:
                    B = wb.iterativeBuildUpRinv(B, xd[bx, p + T - 1], M, L)
                    B = wb.iterativeBuildDownRinv(B, xd[bx, p - 1], M, L)
                ria = Ns * T * B.sum(axis=1)
                aria = ria.sum()
                g = np.array([xd[bx, p + K, i:i + Ns].sum() / Ns for i in range(L)])
                w[bx, p] = ria / aria
                z[bx, p] = np.sum(w[bx, p].conj() * g)
                P[bx, p] = 1.0 / aria.real
    out["slide_params"] = np.array(WOOD_SLIDE, dtype=np.float64)
    out["slide_x"], out["slide_z"], out["slide_P"], out["slide_w"] = x, z, P, w
    return out


# getCaponAllC.pyx (the all-options CPU Capon), (Nx, Ny, M, L, K, d, seed):
# forward-backward averaging in element space with its default Cholesky solver
ALL_FB_CASES = [(2, 24, 16, 8, 1, 0.01, 30), (2, 30, 32, 16, 1, 0.01, 31), (1, 20, 24, 12, 2, 0.05, 32)]
# a general subspace V: (Nx, Ny, M, L, K, d, Nb, seed)
ALL_V_CASE = (2, 24, 16, 8, 1, 0.01, 4, 33)


def _x(Nx, Ny, M, seed):
    rng = np.random.default_rng(seed)
    x = (rng.standard_normal((Nx, Ny, M)) + 1j * rng.standard_normal((Nx, Ny, M))).astype(np.complex64)
    x += (4.0 * np.exp(1j * 0.7 * np.arange(M))[None, None, :]).astype(np.complex64)
    return x


def all_cases() -> dict:
    """Outputs of the reference's getCaponAllC.getCaponCPy.  Its module flags
    select the branches: doFBAvg with the default solver (SOLVE_CHOLESKY on
    the upper triangle it builds); BEAMSPACE with a general V, once through the
    branch that restores R's lower triangle before the transform (SOLVE_NUMPY,
    np.linalg.solve) under both loading orders (DIAGONAL_LOADING_IN_BEAMSPACE),
    and once through the default solver, which transforms an R whose lower
    triangle was never filled (a reference defect, kept as a fixture)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref  # noqa: E402
    ref._prepare()
    import getCaponAllC as A  # noqa: E402
    out = {"fb_cases": np.array(ALL_FB_CASES, dtype=np.float64)}
    for i, (Nx, Ny, M, L, K, d, seed) in enumerate(ALL_FB_CASES):
        x = _x(Nx, Ny, M, seed)
        z, zpow, w = A.getCaponCPy(x.astype(np.complex128), float(d), int(L), int(K), np.array([]), True, False)
        out[f"fb_x{i}"], out[f"fb_z{i}"], out[f"fb_zpow{i}"], out[f"fb_w{i}"] = x, z, zpow, w
    Nx, Ny, M, L, K, d, Nb, seed = ALL_V_CASE
    x = _x(Nx, Ny, M, seed)
    rng = np.random.default_rng(seed + 100)
    V = (rng.standard_normal((Nb, L)) + 1j * rng.standard_normal((Nb, L))) / 4
    out["v_case"] = np.array(ALL_V_CASE, dtype=np.float64)
    out["v_x"], out["v_V"] = x, V
    saved = (A.BEAMSPACE, A.SOLVE_NUMPY, A.SOLVE_CHOLESKY, A.DIAGONAL_LOADING_IN_BEAMSPACE)
    try:
        A.BEAMSPACE = True
        for tag, numpy_solve, in_bs in (("full_bsload", True, True), ("full_elload", True, False),
                                        ("upper_bsload", False, True)):
            A.SOLVE_NUMPY, A.SOLVE_CHOLESKY, A.DIAGONAL_LOADING_IN_BEAMSPACE = numpy_solve, not numpy_solve, in_bs
            z, zpow, w = A.getCaponCPy(x.astype(np.complex128), float(d), L, K, V, False, False)
            out[f"v_{tag}_z"], out[f"v_{tag}_w"] = z, w[..., :Nb]   # beamspace weights, Nb of the L slots
    finally:
        A.BEAMSPACE, A.SOLVE_NUMPY, A.SOLVE_CHOLESKY, A.DIAGONAL_LOADING_IN_BEAMSPACE = saved
    return out


# LCA window selection: (Ny, Nx, Nw, seed) x filters
LCA_SHAPES = [(20, 13, 5, 40), (16, 16, 4, 41)]
LCA_FILTERS = [np.ones((1, 1)), np.ones((5, 1)), np.ones((3, 3)), np.array([[0.5, 1.0, 0.5]]).T,
               np.array([[0.6, 0.9, 0.7], [1.0, 0.8, 0.5], [0.9, 1.0, 0.6], [0.7, 0.5, 1.0], [0.8, 0.6, 0.9]])]


def lca_cases() -> dict:
    """Outputs of the reference's lcac.lca (lcac.py) and lcacx.lca (lcacx.pyx)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref  # noqa: E402
    ref._prepare()
    import lcac  # noqa: E402
    import lcacx  # noqa: E402
    out = {"shapes": np.array(LCA_SHAPES), "nfilters": np.array(len(LCA_FILTERS))}
    for j, wrf in enumerate(LCA_FILTERS):
        out[f"wrf{j}"] = wrf
    for i, (Ny, Nx, Nw, seed) in enumerate(LCA_SHAPES):
        rng = np.random.default_rng(seed)
        Z = rng.standard_normal((Ny, Nx, Nw)) + 1j * rng.standard_normal((Ny, Nx, Nw))
        out[f"Z{i}"] = Z
        for j, wrf in enumerate(LCA_FILTERS):
            r = lcac.lca(Z, np.asarray(wrf, float))
            rx = lcacx.lca(Z, np.asarray(wrf, float))
            out[f"img{i}_{j}"], out[f"win{i}_{j}"] = np.asarray(r[0]), np.asarray(r[1])
            out[f"ximg{i}_{j}"], out[f"xwin{i}_{j}"] = np.asarray(rx[0]), np.asarray(rx[1])
    return out


# time-domain steering: tdib_oracle.scenario arguments
TDIB_CASES = [dict(seed=50, n_h=6, n_s=400, n_x=3, n_y=40), dict(seed=51, n_h=16, n_s=900, n_x=4, n_y=120)]


def tdib_cases() -> dict:
    """Outputs of the reference's tdibC.tdib (tdibC.pyx:9-67, run as Python)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref  # noqa: E402
    import tdib_oracle  # noqa: E402
    ref._prepare()
    import tdibC  # noqa: E402
    out = {"ncases": np.array(len(TDIB_CASES))}
    for i, kw in enumerate(TDIB_CASES):
        sc = tdib_oracle.scenario(**kw)
        if i == 0:
            sc["yarr"][:, -3:] = 400.0   # a few pixels beyond the time axis: NaN
        for k, v in sc.items():
            out[f"{k}{i}"] = np.asarray(v)
        out[f"image{i}"] = tdibC.tdib(sc["mfdata"].astype(np.complex128), sc["mtaxe"], sc["x_r"], sc["D"],
                                      sc["c"], sc["fc"], sc["xarr"], sc["yarr"])
    return out


def main() -> None:
    np.savez_compressed(os.path.join(HERE, "linalg_known_answers.npz"), **known_answers())
    np.savez_compressed(os.path.join(HERE, "capon_ref_cases.npz"), **ref_cases())
    np.savez_compressed(os.path.join(HERE, "woodbury_ref_cases.npz"), **woodbury_cases())
    np.savez_compressed(os.path.join(HERE, "capon_all_ref_cases.npz"), **all_cases())
    np.savez_compressed(os.path.join(HERE, "lca_ref_cases.npz"), **lca_cases())
    np.savez_compressed(os.path.join(HERE, "tdib_ref_cases.npz"), **tdib_cases())
    for f in ("linalg_known_answers.npz", "capon_ref_cases.npz", "woodbury_ref_cases.npz",
              "capon_all_ref_cases.npz", "lca_ref_cases.npz", "tdib_ref_cases.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)), "bytes")


if __name__ == "__main__":
    main()
