"""Loader for the reference's own CPU Capon path compiled by ``oracle/build_ref.py``.

Test infrastructure only (the checker and the CPU baseline), never the product.

``load()`` returns the module ``getCaponC`` (reference
framework/beamformer/capon/getCaponC.pyx) whose ``getCaponCPy(Xd, regCoef, L,
Navg, V, doFBAvg, verbose)`` returns ``[z, zPow, w]`` in complex128, and
``load_linalg()`` returns ``(matrixDecompc, linearSolvec)``.
"""
from __future__ import annotations

import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(HERE, "_ref", "pkg")


def _numpy_aliases() -> None:
    # numpy 2 removed the builtin aliases the reference modules use at import
    # time (linearSolvec.pyx:23-24, matrixDecompc.pyx:14-15, woodburyc.pyx:12-13).
    import numpy as np
    for name, val in (("complex", complex), ("float", float), ("int", int)):
        if name not in np.__dict__:
            setattr(np, name, val)


def available() -> bool:
    return os.path.isdir(PKG) and any(
        f.startswith("getCaponC") and f.endswith(".so") for f in os.listdir(PKG))


def _prepare() -> None:
    if not available():
        raise ImportError("reference CPU path not built: run `python oracle/build_ref.py`")
    _numpy_aliases()
    if PKG not in sys.path:
        sys.path.insert(0, PKG)


def load():
    _prepare()
    import getCaponC  # noqa: E402
    return getCaponC


def load_linalg():
    _prepare()
    from framework.linalg import linearSolvec, matrixDecompc  # noqa: E402
    return matrixDecompc, linearSolvec
