"""Build the lcpgrid shared library (CUDA kernels + C ABI) in-tree.

    python -m lcpgrid.build            (from lcpaodft.jl_gb300/)

compiles every translation unit of ``csrc/`` for sm_103a in parallel and links
``lcpgrid/liblcpgrid.so``.  No CMake; nvcc and g++ only.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)                 # lcpaodft.jl_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG_DIR, "liblcpgrid.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _cuda_root(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def sources():
    out = []
    for name in sorted(os.listdir(CSRC)):
        if name.endswith((".cu", ".cpp")):
            out.append(os.path.join(CSRC, name))
    return out


def _compile(src, nvcc, verbose):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if src.endswith(".cu"):
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-pthread",
               "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
    else:
        # no FMA contraction: the sphere lists' distance tests round like the
        # reference's and the device build's
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-pthread", "-I", INCLUDE, "-I", CSRC,
               "-I", os.path.join(_cuda_root(nvcc), "include"), "-c", src, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    return src, obj, res


def build(verbose=False, force=False):
    """Compile and link; returns the library path.  Raises on failure."""
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "lcpgrid.h"))
    newest = max(os.path.getmtime(p) for p in srcs + headers + [__file__])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) > newest:
        return LIB
    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda s: _compile(s, nvcc, verbose), srcs))
    objs = []
    for src, obj, res in results:
        if verbose and res.stderr:
            sys.stderr.write(res.stderr)
        if res.returncode != 0:
            raise RuntimeError("compilation of %s failed:\n%s%s" % (src, res.stdout, res.stderr))
        objs.append(obj)
    cuda_lib = os.path.join(_cuda_root(nvcc), "lib64")
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-L", cuda_lib, "-lcudart",
           "-Xlinker", "-rpath=" + cuda_lib]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (res.stdout, res.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
