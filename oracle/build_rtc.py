"""Builds the reference's RealTimeCapon GPU library (its own sources, sm_103a)
into oracle/_ref/librtc.so, for timing beside this project's kernels.

TEST/BENCHMARK INFRASTRUCTURE ONLY -- the product never loads it.

Where the reference tree is present, `stage()` places the library's source
files (RealTimeCapon/*.cpp|*.cu|*.h|*.cuh, framework/lib printit + Complex.h,
cuda/include helpers) under oracle/_ref/rtc_src/ (git-ignored) so that the
build can run on a machine without the reference tree; `build()` compiles the
staged files with nvcc plus oracle/rtc_entry.cpp.  Shims (compiler flags only,
the sources are unchanged): cudaThreadSynchronize is mapped to
cudaDeviceSynchronize (removed from CUDA 12+).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference tree: $COS_REFERENCE_ROOT, else a checkout beside this repository
REF = os.environ.get("COS_REFERENCE_ROOT", os.path.join(os.path.dirname(HERE), "..", "reference"))
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "rtc_src")
LIB = os.path.join(OUT, "librtc.so")

RTC_FILES = ["Capon.cpp", "Capon.h", "ICapon.h", "BuildR.cpp", "BuildR.h", "IBuildR.h", "Solver.cpp", "Solver.h",
             "ISolver.h", "CudaUtils.cpp", "CudaUtils.h", "capon_kernel.cu", "capon_kernel.cuh", "buildR_kernel.cu",
             "buildR_kernel.cuh", "nvidia_solve.cu", "nvidia_solve.h", "operations.h", "solver3x3_kernel.cu",
             "solver3x3_kernel.cuh", "solver1x1_kernel.cu", "solver1x1_kernel.cuh", "sliding_beamspace_kernel.cu",
             "sliding_beamspace_kernel.cuh", "cudaConfig.h"]
LIB_FILES = ["printit.cpp", "printit.h", "Complex.h"]
INC_FILES = ["cutil_math.h", "exception.h", "sdkHelper.h", "stopwatch_functions.h", "string_helper.h"]
UNITS = ["Capon.cpp", "BuildR.cpp", "CudaUtils.cpp", "Solver.cpp", "printit.cpp", "capon_kernel.cu",
         "buildR_kernel.cu", "nvidia_solve.cu", "solver3x3_kernel.cu", "solver1x1_kernel.cu",
         "sliding_beamspace_kernel.cu"]


def stage() -> bool:
    rtc = os.path.join(REF, "framework", "beamformer", "capon", "RealTimeCapon")
    if not os.path.isdir(rtc):
        return os.path.isdir(SRC)
    os.makedirs(SRC, exist_ok=True)
    for d, names in ((rtc, RTC_FILES), (os.path.join(REF, "framework", "lib"), LIB_FILES),
                     (os.path.join(REF, "cuda", "include"), INC_FILES)):
        for n in names:
            shutil.copy2(os.path.join(d, n), os.path.join(SRC, n))
    return True


def build(verbose: bool = False) -> str | None:
    if not stage():
        return None
    srcs = [os.path.join(SRC, u) for u in UNITS] + [os.path.join(HERE, "rtc_entry.cpp")]
    newest = max(os.path.getmtime(s) for s in srcs)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    objdir = os.path.join(OUT, "rtc_obj")
    os.makedirs(objdir, exist_ok=True)
    flags = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
             "-DcudaThreadSynchronize=cudaDeviceSynchronize", "-I" + SRC, "-w"]
    procs, objs = [], []
    for s in srcs:
        o = os.path.join(objdir, os.path.basename(s) + ".o")
        objs.append(o)
        procs.append(subprocess.Popen(["nvcc", *flags, "-x", "cu" if s.endswith(".cu") else "c++", "-c", s, "-o", o],
                                      stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
    for p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + out[-3000:])
        if verbose and out.strip():
            print(out)
    tmp = LIB + ".tmp"
    subprocess.run(["nvcc", "-shared", "-gencode", "arch=compute_103a,code=sm_103a", *objs, "-lcublas", "-o", tmp],
                   check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
