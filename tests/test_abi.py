"""The C-ABI library: it builds, loads, exports every symbol include/cos_capon.h
declares, and rejects NULL handles without touching a GPU.  CPU only."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "cos_capon.h")


def _declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(cos_capon_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def libmod():
    from cos_gb300 import build
    build.build()
    from cos_gb300 import _lib
    return _lib


def test_header_declares_expected_entry_points(libmod):
    assert _declared() == sorted(libmod.EXPORTS)


def test_library_exports_every_declared_symbol(libmod):
    lib = C.CDLL(libmod.LIB_PATH)
    for name in _declared():
        assert hasattr(lib, name), name


def test_status_codes_match_cuda_runtime_numbers(libmod):
    # the reference returns cudaError_t values (Capon.cpp:101, 122)
    assert libmod.ERR_LAUNCH == 719 and libmod.ERR_OUT_OF_MEMORY == 32
    for code in (0, 1, 32, 719, 801, 909):
        assert libmod.status_string(code)


def test_null_context_is_rejected(libmod):
    lib = libmod.lib
    assert lib.cos_capon_destroy(None) == libmod.ERR_INVALID_VALUE
    assert lib.cos_capon_device_status(None) == libmod.ERR_INVALID_VALUE
    assert lib.cos_capon_get_capon(None, None, None, None, None, 0.01, 8, 1, 16, 2, 10, 0) == \
        libmod.ERR_INVALID_VALUE
    assert lib.cos_capon_run(None, None, 0, None, None) == libmod.ERR_INVALID_VALUE
    assert lib.cos_capon_solve(None, None, None, None, 3, 1, 0, 0, 0) == libmod.ERR_INVALID_VALUE
    assert lib.cos_capon_create(None) == libmod.ERR_INVALID_VALUE


def test_create_without_gpu_fails_cleanly(libmod):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    rc = libmod.lib.cos_capon_create(C.byref(h))
    assert rc != 0 and not h.value


def test_cxx_shim_compiles():
    """include/cos_capon.hpp (the ICapon-compatible C++ class) compiles against
    the C header with a plain C++ compiler."""
    import subprocess
    import tempfile
    src = '#include "cos_capon.hpp"\nint main(){ Capon c; (void)c; return 0; }\n'
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "t.cpp")
        open(f, "w").write(src)
        p = subprocess.run(["g++", "-std=c++11", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), f],
                           capture_output=True, text=True)
        assert p.returncode == 0, p.stderr


def test_new_entry_points_reject_null_context_without_touching_the_gpu():
    """The steering, LCA and subspace calls validate their arguments first."""
    import ctypes as C
    from cos_gb300 import _lib
    x = np.zeros(8, np.complex64)
    d = np.zeros(8)
    assert _lib.lib.cos_capon_tdib(None, x.ctypes.data, 2, 4, 0.0, 1.0, d.ctypes.data, d.ctypes.data, 1500.0,
                                   1e5, d.ctypes.data, d.ctypes.data, 2, 2, x.ctypes.data, None, 0,
                                   None) == _lib.ERR_INVALID_VALUE
    assert _lib.lib.cos_capon_lca(None, x.ctypes.data, 2, 2, 2, d.ctypes.data, 1, 1, x.ctypes.data, None, 0,
                                  None) == _lib.ERR_INVALID_VALUE
    assert _lib.lib.cos_capon_get_capon_subspace(None, x.ctypes.data, None, None, x.ctypes.data, x.ctypes.data,
                                                 0.01, 4, 1, 8, 1, 4, 2, None) == _lib.ERR_INVALID_VALUE


def test_steering_time_axis_must_be_uniform():
    import pytest
    from cos_gb300 import tdib
    assert tdib._axis(np.arange(10) * 0.5 + 2.0) == (2.0, 0.5)
    with pytest.raises(ValueError):
        tdib._axis(np.array([0.0, 1.0, 3.0]))
    with pytest.raises(ValueError):
        tdib._axis(np.array([1.0]))


def test_struct_layouts_match_the_header(libmod, tmp_path):
    # sizeof / offsetof of every struct of the header, compiled by the C
    # compiler, against the ctypes mirrors the Python side passes
    structs = {"cos_capon_opts": libmod.Opts, "cos_capon_frame": libmod.Frame,
               "cos_capon_adjoint": libmod.Adjoint}
    lines = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void) {"]
    for cname, cls in structs.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["return 0;", "}"]
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text("\n".join(lines))
    import subprocess
    subprocess.run(["gcc", "-std=c11", str(src), "-o", str(exe)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], check=True, capture_output=True,
                                                 text=True).stdout.splitlines())
    for cname, cls in structs.items():
        assert int(got[cname]) == C.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(cls, fname).offset, f"{cname}.{fname}"
