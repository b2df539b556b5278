"""Build the pplacer_gb300 CUDA library in-tree for sm_103a.

    python -m pplacer_gb300.build          # -> pplacer_gb300/_build/libpplacer_gb300.so

Each .cu file is compiled by its own nvcc process (in parallel), then linked
into one shared library exporting the C ABI of include/pplacer_gb300.h.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libpplacer_gb300.so")
SOURCES = ["dropin.cu", "engine.cu", "noalloc.cu", "tc.cu"]
# The drop-in keeps linear_c.c's unfused multiply-add arithmetic so that its
# FP64 results equal the reference's to the last bit where the summation order
# is the same.
EXTRA = {"dropin.cu": ["-fmad=false"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pplacer_gb300")
    return cand


def _compile(src, verbose_ptxas=False):
    obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-c",
           os.path.join(CSRC, src), "-o", obj, "-I", os.path.join(ROOT, "include")]
    cmd += EXTRA.get(src, [])
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def build(force=False, verbose_ptxas=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "pplacer_gb300.h")]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(s) <= t for s in srcs):
            return LIB
    with ThreadPoolExecutor(len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose_ptxas), SOURCES))
    objs = [o for o, _ in results]
    if verbose_ptxas:
        for _, log in results:
            sys.stderr.write(log)
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
