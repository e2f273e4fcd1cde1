"""Builds the engine's shared library lib/libg4gpu.so for sm_103a (GB300).

Each translation unit is compiled in parallel; nothing else is needed than nvcc
and g++. The library is built in-tree and is what include/g4gpu.h describes.

  kernels_plain.cu   FP64 kernels, compiled with --fmad=false (reference rounding)
  kernels_mixed.cu   mixed-precision kernels
  kernels_util.cu    layout conversions
  kernels_sort.cu    one4one sorting of a window (--fmad=false: the reference's rounding)
  kernels_fft.cu     FFT field solver (mixed-radix Stockham, FP64 and FP32)
  kernels_mlp.cu     BF16 tensor-core MLP of the learned closure (training and inference)
  kernels_closure.cu per-slice features and corrections of the learned closure
  g4gpu_api.cpp      C ABI, host bookkeeping (-ffp-contract=off)
  host_loading.cpp   bit-exact host loading (-ffp-contract=off)
  g4gpu_learned.cpp  learned closure: MLP object, features / corrections, coarse-step driver
  g4gpu_dpi.cpp      diagnostic plugins (DPI) of the reference's plugin interface, fed from the engine
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "_build")
LIB_DIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIB_DIR, "libg4gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _units():
    cu_common = ["nvcc", "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
                 "-Xcompiler", "-ffp-contract=off", "-I", INC, "-I", CSRC] + ARCH
    cxx_common = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-I", INC, "-I", CSRC,
                  "-I", os.path.join(_cuda_home(), "include")]
    return [
        ("kernels_plain.cu", cu_common + ["--fmad=false"]),
        # the mixed form tolerates approximate FP32 division, square root and
        # sin/cos (errors ~1e-7 relative, far below its 1 % target)
        ("kernels_mixed.cu", cu_common + ["-use_fast_math"]),
        ("kernels_util.cu", cu_common),
        ("kernels_sort.cu", cu_common + ["--fmad=false"]),
        ("kernels_fft.cu", cu_common),
        ("kernels_mlp.cu", cu_common),
        ("kernels_closure.cu", cu_common + ["-use_fast_math"]),
        ("g4gpu_api.cpp", cxx_common),
        ("host_loading.cpp", cxx_common + ["-pthread"]),
        ("host_wake.cpp", cxx_common + ["-pthread"]),
        ("h5_writer.cpp", cxx_common),
        ("g4gpu_learned.cpp", cxx_common),
        ("g4gpu_dpi.cpp", cxx_common),
    ]


def _compile(src, cmd):
    out = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    full = cmd + ["-c", os.path.join(CSRC, src), "-o", out]
    r = subprocess.run(full, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile {src} failed:\n{' '.join(full)}\n{r.stdout}\n{r.stderr}")
    return out


def _stale(outputs, inputs):
    if not all(os.path.exists(o) for o in outputs):
        return True
    t = min(os.path.getmtime(o) for o in outputs)
    return any(os.path.getmtime(i) > t for i in inputs)


def build(force=False, verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    srcs = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INC, "g4gpu.h"),
                                                                os.path.abspath(__file__)]
    if not force and not _stale([LIB], srcs):
        return LIB
    units = _units()
    with cf.ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(lambda u: _compile(*u), units))
    tmp = LIB + ".tmp"
    cmd = ["nvcc", "-shared", "-o", tmp] + ARCH + objs + ["-lpthread", "-ldl"]
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
