"""The C++ drop-in on the GPU: a program written against the reference's
RealTimeCapon classes (Capon::getCapon, BuildR::getR, Solver::solve, the
calls of apps/RealTimeCaponTest/App.cpp) is compiled against
include/cos_capon.hpp, linked to libcos_capon.so and run; its z, w, R, the
stage R and the solver's x equal the ctypes path's outputs bit for bit."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cxx_program_matches_ctypes_path(tmp_path):
    from cos_gb300 import _lib, capon, synth
    Nx, Nz, M, L, K, d, nsys = 4, 96, 64, 32, 2, 0.01, 7
    x = synth.cube(Nz, Nx, M, [10.0, 5.0], seed=41)
    exe = tmp_path / "app"
    libdir = os.path.dirname(_lib.LIB_PATH)
    p = subprocess.run(["g++", "-std=c++11", "-O2", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cxx_dropin_app.cpp"), "-o", str(exe),
                        "-L", libdir, "-lcos_capon", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    x.tofile(tmp_path / "cube.bin")
    r = subprocess.run([str(exe), str(tmp_path / "cube.bin"), str(tmp_path), str(Nx), str(Nz), str(M), str(L),
                        str(K), repr(d), str(nsys)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.split() == ["0", "0", "0"], r.stdout

    npy = Nz - 2 * K
    def load(name, shape):
        return np.fromfile(tmp_path / name, dtype=np.complex64).reshape(shape)
    z_c, w_c = load("z.bin", (Nx, npy)), load("w.bin", (Nx, npy, L))
    R_c, Rb_c = load("R.bin", (Nx, npy, L, L)), load("Rb.bin", (Nx, npy, L, L))
    xs_c = load("xs.bin", (nsys, L))

    z = np.zeros((Nx, npy), np.complex64)
    w = np.zeros((Nx, npy, L), np.complex64)
    R = np.zeros((Nx, npy, L, L), np.complex64)
    assert capon.Capon().getCapon(z, w, R, x, d, L, K, M, Nx, Nz, 0) == 0
    Rb = np.zeros_like(R)
    assert capon.BuildR().getR(Rb, x, d, L, K, M, Nx, Nz, 0) == 0
    xs = np.zeros((nsys, L), np.complex64)
    A = np.ascontiguousarray(Rb.reshape(-1, L, L)[:nsys])
    assert capon.Solver().solve(xs, A, np.ones((nsys, L), np.complex64), L, nsys) == 0
    for name, a, b in (("z", z_c, z), ("w", w_c, w), ("R", R_c, R), ("Rb", Rb_c, Rb), ("xs", xs_c, xs)):
        assert np.array_equal(a, b), name
