"""Build libmlau_gb300.so (sm_103a) in-tree with nvcc.

Translation units compile in parallel, each with one ``-gencode`` for
sm_103a.  The plain FP64 kernels are built with ``--fmad=false`` so that no
multiply-add is contracted: their arithmetic must match the reference's
(compiled without FMA) bit for bit.  The FP32-split kernels use FMA and fast
FP32 division/square root.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libmlau_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE]
EXACT = ["--fmad=false"]
FAST32 = ["--fmad=true", "--prec-div=false", "--prec-sqrt=false", "--ftz=true"]

UNITS = {
    "plain3d.cu": EXACT,
    "plain2d.cu": EXACT,
    "plain1d.cu": EXACT,
    "cfl.cu": EXACT,
    "split3d.cu": FAST32,
    "api.cu": EXACT,
    "peaks.cu": EXACT,
    "noalloc1d.cu": EXACT,
    "batch2d.cu": EXACT,
    "batch2d_split.cu": FAST32,
    "batch2d_plain.cu": EXACT,
    "batch1d_plain.cu": EXACT,
    "dataio.cu": EXACT,
    "diff2d.cu": EXACT,
    "cxx_linkage.cpp": [],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmlau_gb300.so")


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + [
        os.path.join(INCLUDE, "mlau_gb300.h")]


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    cc = nvcc()
    hdrs = _headers()
    objs, work = [], []
    for src, extra in UNITS.items():
        path = os.path.join(CSRC, src)
        obj = os.path.join(OBJDIR, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path, __file__] + hdrs):
            if src.endswith(".cpp"):
                cmd = ["g++", "-O2", "-fPIC", "-std=c++17", "-c", path, "-o", obj]
            else:
                cmd = [cc, *ARCH, *COMMON, *extra, "-c", path, "-o", obj]
            work.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    with ThreadPoolExecutor(jobs or min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(run, work))
    if work or force or _stale(LIB, objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-lpthread",
               "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        os.replace(tmp, LIB)
    return LIB


def ptxas_report(src: str = "plain3d.cu") -> str:
    """Registers/spills per kernel (-Xptxas -v) of one translation unit."""
    path = os.path.join(CSRC, src)
    cmd = [nvcc(), *ARCH, *COMMON, *UNITS[src], "-Xptxas", "-v", "-c", path, "-o", os.devnull]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r.stdout + r.stderr


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
