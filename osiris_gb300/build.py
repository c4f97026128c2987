"""Build recipe of the native library (no cmake): nvcc for sm_103a, parallel per-file compile.

    python -m osiris_gb300.build          # or osiris_gb300.build.build()

Outputs (in-tree, git-ignored):
    osiris_gb300/libosiris_gb300.so          the C ABI of include/osiris_gb300.h
    osiris_gb300/libosiris_gb300_single.so   reference-named drop-in symbols, REAL = float
    osiris_gb300/libosiris_gb300_double.so   reference-named drop-in symbols, REAL = double
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libosiris_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no implicit multiply-add contraction (explicit fma only), IEEE div/sqrt
NVFLAGS = ["-std=c++17", "-O3", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr", "-I", ROOT]

# The tiled (mixed-precision) Boris kernels use the approximate single-precision division and
# square root (at most 2 ulp): measured 4% faster on the two-stream push, inside the mixed
# engine's 1e-5 parity.  The drop-in and plain kernels keep IEEE rounding (bit-identical to the
# reference), and so does the exact pusher: its k^2 = (inv1 + sqrt(inv1^2 + 4 inv2^2)) / 2 needs
# the correctly rounded square root to stay >= 0 when E.B = 0 and |B| > |E|.
FAST_DIV = ["-prec-div=false", "-prec-sqrt=false"]
EXTRA = {"tiled.cu": FAST_DIV, "batch_push.cu": FAST_DIV}

SOURCES = ["push_plain.cu", "fields.cu", "tiled.cu", "tiled_exact.cu", "tiled_vay.cu", "tiled_hc.cu",
           "tiled_fullrot.cu", "tiled_euler.cu", "tiled_condvay.cu",
           "batch_push.cu", "batch.cu",
           "sim.cu", "capi.cu", "noalloc.cu",
           "loader.cpp", "laser.cpp"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _compile(src: str, verbose: bool) -> str:
    out = os.path.join(OBJ, os.path.basename(src) + ".o")
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(ROOT, "include", "osiris_gb300.h")]
    if _newer(out, deps):
        return out
    cmd = [nvcc()] + ARCH + NVFLAGS + EXTRA.get(src, []) + ["-c", os.path.join(CSRC, src), "-o", out]
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-x", "c++"] + NVFLAGS + ["-c", os.path.join(CSRC, src), "-o", out]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{r.stdout}\n{r.stderr}")
    return out


def build(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if not _newer(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lrt",
                                                                  "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    shim_src = os.path.join(CSRC, "fortran_shim.c")
    for prec, flag in (("single", "-DOSG_PRECISION_SINGLE"), ("double", "-DOSG_PRECISION_DOUBLE")):
        shim = os.path.join(HERE, f"libosiris_gb300_{prec}.so")
        if not _newer(shim, [shim_src, LIB, os.path.join(ROOT, "include", "osiris_gb300_fortran.h")]):
            cmd = ["gcc", "-O2", "-fPIC", "-shared", flag, "-I", ROOT, "-o", shim, shim_src,
                   "-L", HERE, "-losiris_gb300", "-Wl,-rpath,$ORIGIN"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"shim build failed\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
