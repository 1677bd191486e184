"""Build the reference's own CPU Capon path (Cython, FP64) into ``oracle/_ref/``.

Test infrastructure only: the compiled modules are the *checker* for the CUDA
path and the CPU baseline of ``bench.py``; nothing in the product imports them.

Two stages:

``cythonize``  (needs the reference sources and Cython; run where both exist)
    Copies the few source files of the path into ``oracle/_ref/src`` and applies
    the minimal shims they need under Cython 3 / numpy 2, then generates C++:

    * ``framework/linalg/matrixDecompc.pyx``  -- ``cholesky`` (upper U, UᴴU = A)
    * ``framework/linalg/linearSolvec.pyx``   -- ``solveCholesky``,
      ``forwardSolve``, ``backtrackSolve``
    * ``framework/linalg/woodburyc.pyx``      -- cimported by getCaponC (unused
      by the default solver, but the module must exist)
    * ``framework/beamformer/capon/getCaponC.pyx`` -- ``getCaponCPy``
    * ``framework/lib/Complex.{pxd,h}``       -- the POD complex type

    Shims (applied to the copies only, never to the reference):
    1. drop ``cimport cython.array`` (getCaponC.pyx:44; the module no longer
       exists in Cython 3 and is unused);
    2. ``ctypedef np.int_t ITYPE_t`` -> ``ctypedef long ITYPE_t``
       (getCaponC.pyx:58; ``np.int_t`` was removed from numpy 2's pxd);
    3. at import time ``np.complex/np.float/np.int`` are restored as aliases of
       the builtins (numpy 2 removed them; used at linearSolvec.pyx:23-24,
       matrixDecompc.pyx:14-15) -- see ``oracle/ref.py``.

``compile``  (needs g++, Python headers and numpy; runs here and on the GPU host)
    Compiles the generated C++ into importable extension modules under
    ``oracle/_ref/pkg``.  The generated C++ is plain text and travels with the
    repository snapshot, so the GPU host (which has no Cython) only runs this
    stage.

Usage:  python oracle/build_ref.py [cythonize] [compile]   (default: both, as possible)
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference tree: $COS_REFERENCE_ROOT, else a checkout beside this repository
REF_ROOT = os.environ.get("COS_REFERENCE_ROOT", os.path.join(os.path.dirname(HERE), "..", "reference"))
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
PKG = os.path.join(OUT, "pkg")

# (source path within the reference, destination path within src/)
FILES = [
    ("framework/linalg/matrixDecompc.pyx", "framework/linalg/matrixDecompc.pyx"),
    ("framework/linalg/matrixDecompc.pxd", "framework/linalg/matrixDecompc.pxd"),
    ("framework/linalg/linearSolvec.pyx", "framework/linalg/linearSolvec.pyx"),
    ("framework/linalg/linearSolvec.pxd", "framework/linalg/linearSolvec.pxd"),
    ("framework/linalg/woodburyc.pyx", "framework/linalg/woodburyc.pyx"),
    ("framework/linalg/woodburyc.pxd", "framework/linalg/woodburyc.pxd"),
    ("framework/beamformer/capon/getCaponC.pyx", "getCaponC.pyx"),
    ("framework/lib/Complex.pxd", "Complex.pxd"),
    ("framework/lib/Complex.h", "Complex.h"),
    # the "next" rows of the path: the all-options CPU Capon (forward-backward
    # averaging, general subspace V), the LCA window selection, the steering
    ("framework/beamformer/capon/getCaponAllC.pyx", "getCaponAllC.pyx"),
    ("framework/beamformer/lca/lcac.py", "lcac.pyx"),
    ("framework/beamformer/lca/lcacx.pyx", "lcacx.pyx"),
    ("framework/beamformer/delay/tdibC.pyx", "tdibC.py"),
]

# modules: (pyx relative to src, fully qualified module name)
MODULES = [
    ("framework/linalg/matrixDecompc.pyx", "framework.linalg.matrixDecompc"),
    ("framework/linalg/linearSolvec.pyx", "framework.linalg.linearSolvec"),
    ("framework/linalg/woodburyc.pyx", "framework.linalg.woodburyc"),
    ("getCaponC.pyx", "getCaponC"),
    ("getCaponAllC.pyx", "getCaponAllC"),
    ("lcac.pyx", "lcac"),
    ("lcacx.pyx", "lcacx"),
]
# pure-Python reference modules, shimmed copies imported as they are
PY_MODULES = [("tdibC.py", "tdibC")]


def _shim(dst_rel: str, text: str) -> str:
    """Shims applied to the staged copies (never to the reference tree):
    numpy-2 type names, the missing framework.mynumpy (a numpy wrapper), the
    unused GPU BuildR cimport and MKL spline import, Python 2 prints in the
    pure-Python module."""
    if dst_rel in ("getCaponC.pyx", "getCaponAllC.pyx", "lcac.pyx", "lcacx.pyx"):
        text = text.replace("cimport cython.array\n", "\n")
        text = re.sub(r"ctypedef\s+np\.int_t\s+ITYPE_t", "ctypedef long ITYPE_t", text)
        text = text.replace("import framework.mynumpy as np", "import numpy as np")
    if dst_rel == "getCaponAllC.pyx":
        # cimported but never used on the CPU path (getCaponAllC.pyx:25)
        text = text.replace("from framework.beamformer.capon.RealTimeCapon.BuildR cimport BuildR", "")
    if dst_rel == "tdibC.py":
        text = text.replace("from framework.mynumpy import pi", "from numpy import pi")
        text = text.replace("import framework.mynumpy as np", "import numpy as np")
        text = text.replace("from framework.lib.mkl.mklUnivariateSplineC import mklcUnivariateSplineC", "")
        text = re.sub(r"print '([^']*)'", r"print('\1')", text)
    return text


def cythonize() -> None:
    if not os.path.isdir(REF_ROOT):
        raise FileNotFoundError(f"reference sources not found at {REF_ROOT}")
    import Cython  # noqa: F401  (fails loudly if Cython is absent)

    os.makedirs(os.path.join(SRC, "framework", "linalg"), exist_ok=True)
    for pkg_dir in ("framework", "framework/linalg"):
        open(os.path.join(SRC, pkg_dir, "__init__.py"), "w").close()
    for src_rel, dst_rel in FILES:
        with open(os.path.join(REF_ROOT, src_rel), "r", encoding="latin-1") as f:
            text = f.read()
        with open(os.path.join(SRC, dst_rel), "w", encoding="latin-1") as f:
            f.write(_shim(dst_rel, text))
    for pyx, _mod in MODULES:
        cmd = [sys.executable, "-m", "cython", "-2", "--cplus", "-I", SRC,
               "-I", os.path.join(SRC, "framework", "linalg"), pyx]
        subprocess.run(cmd, cwd=SRC, check=True)


def _compile_one(pyx: str, mod: str) -> str:
    import numpy as np

    cpp = os.path.join(SRC, pyx[:-4] + ".cpp")
    if not os.path.exists(cpp):
        raise FileNotFoundError(f"{cpp} missing: run the cythonize stage where Cython exists")
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    out = os.path.join(PKG, *mod.split(".")) + suffix
    os.makedirs(os.path.dirname(out), exist_ok=True)
    cmd = ["g++", "-O2", "-shared", "-fPIC", "-w",
           "-I", sysconfig.get_paths()["include"], "-I", np.get_include(), "-I", SRC,
           cpp, "-o", out]
    subprocess.run(cmd, check=True)
    return out


def compile_modules() -> list[str]:
    for pkg_dir in ("framework", "framework/linalg"):
        os.makedirs(os.path.join(PKG, pkg_dir), exist_ok=True)
        open(os.path.join(PKG, pkg_dir, "__init__.py"), "w").close()
    built = []
    for py, mod in PY_MODULES:
        src = os.path.join(SRC, py)
        if os.path.exists(src):
            shutil.copy2(src, os.path.join(PKG, mod + ".py"))
            built.append(os.path.join(PKG, mod + ".py"))
    mods = [m for m in MODULES if os.path.exists(os.path.join(SRC, m[0][:-4] + ".cpp"))]
    with ThreadPoolExecutor(max_workers=max(1, len(mods))) as ex:
        return built + list(ex.map(lambda m: _compile_one(*m), mods))


def main(argv: list[str]) -> None:
    stages = argv or ["cythonize", "compile"]
    if "cythonize" in stages:
        cythonize()
    if "compile" in stages:
        for p in compile_modules():
            print("built", os.path.relpath(p, HERE))


if __name__ == "__main__":
    main(sys.argv[1:])
