"""Build the in-tree native library ``laml_gb300/_lib/liblaml_gb300.so``.

One nvcc invocation per translation unit (run in parallel), sm_103a only, then
one link.  Host code is plain C++17 with no architecture-specific flags, so
the same recipe builds on x86_64 and aarch64 (Grace).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "liblaml_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["encode.cpp", "pmm_kernels.cu"]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _compile(src, obj, extra):
    cmd = [nvcc(), "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
           "-I" + os.path.join(ROOT, "include"), *ARCH, *extra, "-c",
           os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose=False, extra=()):
    os.makedirs(OUT_DIR, exist_ok=True)
    objs = [os.path.join(OUT_DIR, os.path.splitext(s)[0] + ".o") for s in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(lambda a: _compile(a[0], a[1], list(extra)), zip(SOURCES, objs)))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", *ARCH, "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    for o in objs:
        os.remove(o)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
