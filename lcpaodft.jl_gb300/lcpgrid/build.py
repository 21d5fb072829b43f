"""Build the lcpgrid shared library (CUDA kernels + C ABI) in-tree.

    python -m lcpgrid.build            (from lcpaodft.jl_gb300/)

compiles every translation unit of ``csrc/`` for sm_103a in parallel and links
``lcpgrid/liblcpgrid.so``, and the same sources with LCP_BOUNDS_CHECK (device
bounds checks on every gathered index) into ``lcpgrid/liblcpgrid_check.so``.
No CMake; nvcc and g++ only.
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
# the check build: the same sources with device-side bounds checks
BUILD_CHECK = os.path.join(ROOT, "_build_check")
LIB_CHECK = os.path.join(PKG_DIR, "liblcpgrid_check.so")

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


def _compile(src, nvcc, verbose, outdir, defines):
    obj = os.path.join(outdir, os.path.basename(src) + ".o")
    if src.endswith(".cu"):
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-pthread",
               "--expt-relaxed-constexpr", *defines, "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
    else:
        # no FMA contraction: the sphere lists' distance tests round like the
        # reference's and the device build's
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-pthread", *defines, "-I", INCLUDE,
               "-I", CSRC, "-I", os.path.join(_cuda_root(nvcc), "include"), "-c", src, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    return src, obj, res


def _variants(check):
    out = [(BUILD, LIB, [])]
    if check:
        out.append((BUILD_CHECK, LIB_CHECK, ["-DLCP_BOUNDS_CHECK"]))
    return out


def build(verbose=False, force=False, check=True):
    """Compile and link the library (and, with check, its bounds-check
    build); returns the library path.  Raises on failure."""
    nvcc = _nvcc()
    srcs = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "lcpgrid.h"))
    newest = max(os.path.getmtime(p) for p in srcs + headers + [__file__])
    todo = [(d, lib, defs) for d, lib, defs in _variants(check)
            if force or not os.path.exists(lib) or os.path.getmtime(lib) <= newest]
    if not todo:
        return LIB
    jobs = []
    for outdir, lib, defs in todo:
        os.makedirs(outdir, exist_ok=True)
        jobs += [(src, outdir, defs) for src in srcs]
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda j: _compile(j[0], nvcc, verbose, j[1], j[2]), jobs))
    for src, obj, res in results:
        if verbose and res.stderr:
            sys.stderr.write(res.stderr)
        if res.returncode != 0:
            raise RuntimeError("compilation of %s failed:\n%s%s" % (src, res.stdout, res.stderr))
    cuda_lib = os.path.join(_cuda_root(nvcc), "lib64")
    for outdir, lib, defs in todo:
        objs = [os.path.join(outdir, os.path.basename(src) + ".o") for src in srcs]
        tmp = lib + ".tmp"
        cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-L", cuda_lib, "-lcudart", "-Xlinker", "-rpath=" + cuda_lib]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (res.stdout, res.stderr))
        os.replace(tmp, lib)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
