"""ctypes binding of ``libcos_capon.so`` (the C ABI of ``include/cos_capon.h``).

There is no fallback: if the library is missing or fails to load, importing
this module raises, so a caller can never silently run something else.
"""
from __future__ import annotations

import ctypes as C
import os

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libcos_capon.so")

# status codes (include/cos_capon.h)
SUCCESS = 0
ERR_INVALID_VALUE = 1
ERR_OUT_OF_MEMORY = 32
ERR_LAUNCH = 719
ERR_NOT_SUPPORTED = 801
ERR_TIMEOUT = 909

FORM_FUSED, FORM_PLAIN, FORM_TC_TF32, FORM_TC_BF16X3, FORM_TC_TF32X3 = 0, 1, 2, 3, 4
FORM_SLIDING_INVERSE = 5
FORM_TC_FUSED = 6
LOAD_ELEMENT, LOAD_BEAMSPACE, LOAD_ABSOLUTE = 0, 1, 2
R_REFERENCE, R_NORMALISED = 0, 1
REFINE_NONE, REFINE_ALL, REFINE_ADAPTIVE = 0, 1, 2

# every symbol include/cos_capon.h declares
EXPORTS = (
    "cos_capon_create", "cos_capon_destroy", "cos_capon_get_capon", "cos_capon_get_capon_ex",
    "cos_capon_run", "cos_capon_build_r", "cos_capon_solve", "cos_capon_butler",
    "cos_capon_device_status", "cos_capon_status_string", "cos_capon_run_plain_noalloc",
    "cos_capon_backward", "cos_capon_get_capon_subspace", "cos_capon_tdib", "cos_capon_lca",
)


class Opts(C.Structure):
    _fields_ = [("form", C.c_int), ("loading", C.c_int), ("r_layout", C.c_int), ("refine", C.c_int),
                ("fb", C.c_int), ("segment", C.c_int)]


class Frame(C.Structure):
    _fields_ = [
        ("x", C.c_void_p), ("z", C.c_void_p), ("P", C.c_void_p), ("w", C.c_void_p), ("R", C.c_void_p),
        ("d", C.c_float), ("L", C.c_int), ("K", C.c_int), ("M", C.c_int), ("Nx", C.c_int),
        ("Ny", C.c_int), ("Nb", C.c_int), ("V", C.c_void_p),
    ]


class Adjoint(C.Structure):
    _fields_ = [("x", C.c_void_p), ("w", C.c_void_p), ("gP", C.c_void_p), ("gx", C.c_void_p),
                ("gd", C.c_void_p), ("gtheta", C.c_void_p), ("L", C.c_int), ("K", C.c_int), ("M", C.c_int),
                ("Nx", C.c_int), ("Ny", C.c_int)]


class CaponError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        super().__init__(f"{what}: status {status} ({status_string(status)})" if what else
                         f"status {status} ({status_string(status)})")


def _load() -> C.CDLL:
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(LIB_PATH)
    vp, i, f = C.c_void_p, C.c_int, C.c_float
    sig = {
        "cos_capon_create": [C.POINTER(vp)],
        "cos_capon_destroy": [vp],
        "cos_capon_get_capon": [vp, vp, vp, vp, vp, f, i, i, i, i, i, i],
        "cos_capon_get_capon_ex": [vp, vp, vp, vp, vp, vp, f, i, i, i, i, i, i, C.POINTER(Opts)],
        "cos_capon_run": [vp, C.POINTER(Frame), i, C.POINTER(Opts), vp],
        "cos_capon_build_r": [vp, vp, vp, f, i, i, i, i, i, i, i, i],
        "cos_capon_solve": [vp, vp, vp, vp, i, i, i, i, i],
        "cos_capon_butler": [vp, vp, i, i, i],
        "cos_capon_device_status": [vp],
        "cos_capon_status_string": [i],
        "cos_capon_run_plain_noalloc": [C.POINTER(Frame), vp],
        "cos_capon_backward": [vp, C.POINTER(Adjoint), vp],
        "cos_capon_get_capon_subspace": [vp, vp, vp, vp, vp, vp, f, i, i, i, i, i, i, C.POINTER(Opts)],
        "cos_capon_tdib": [vp, vp, i, i, C.c_double, C.c_double, vp, vp, C.c_double, C.c_double, vp, vp, i, i,
                           vp, vp, i, vp],
        "cos_capon_lca": [vp, vp, i, i, i, vp, i, i, vp, vp, i, vp],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_char_p if name == "cos_capon_status_string" else C.c_int
    return lib


lib = _load()


def status_string(status: int) -> str:
    return lib.cos_capon_status_string(int(status)).decode()


def check(status: int, what: str = "") -> None:
    if status != SUCCESS:
        raise CaponError(status, what)
