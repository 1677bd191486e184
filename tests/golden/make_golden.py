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


def main() -> None:
    np.savez_compressed(os.path.join(HERE, "linalg_known_answers.npz"), **known_answers())
    np.savez_compressed(os.path.join(HERE, "capon_ref_cases.npz"), **ref_cases())
    np.savez_compressed(os.path.join(HERE, "woodbury_ref_cases.npz"), **woodbury_cases())
    for f in ("linalg_known_answers.npz", "capon_ref_cases.npz", "woodbury_ref_cases.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)), "bytes")


if __name__ == "__main__":
    main()
