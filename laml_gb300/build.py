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


def build(verbose=False, extra=(), out=None):
    """Compile and link; ``extra`` are additional nvcc flags (e.g. -D tile
    settings) and ``out`` an alternative library path for such variants."""
    lib = out or LIB
    os.makedirs(os.path.dirname(lib), exist_ok=True)
    tag = os.path.splitext(os.path.basename(lib))[0]
    objs = [os.path.join(os.path.dirname(lib), f"{tag}_{os.path.splitext(s)[0]}.o")
            for s in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(lambda a: _compile(a[0], a[1], list(extra)), zip(SOURCES, objs)))
    tmp = lib + ".tmp"
    cmd = [nvcc(), "-shared", *ARCH, "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    for o in objs:
        os.remove(o)
    if verbose:
        print("built", lib)
    return lib


if __name__ == "__main__":
    args = sys.argv[1:]
    out = None
    if "-o" in args:
        i = args.index("-o")
        out = args[i + 1]
        args = args[:i] + args[i + 2:]
    build(verbose=True, extra=args, out=out)
