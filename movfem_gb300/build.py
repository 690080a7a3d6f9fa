"""Build the CUDA library ``libmovfem_gpu.so`` in-tree with nvcc for sm_103a.

Translation units are compiled in parallel and linked with ``-shared``; the result
lands in ``movfem_gb300/_build/`` (git-ignored).  Rebuilds only when a source is
newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libmovfem_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build movfem_gb300")
    return p


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def host_sources():
    """Host-only translation units (g++, no floating-point contraction)."""
    return sorted(glob.glob(os.path.join(CSRC, "*.cpp")))


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = sources() + host_sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + [
        os.path.join(HERE, "..", "include", "movfem_gpu.h"), __file__]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp,-O2", "--expt-relaxed-constexpr",
                    "-DNDEBUG"]
    objs = []

    host_flags = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-DNDEBUG"]

    def one(src):
        obj = os.path.join(BUILD, os.path.basename(src).rsplit(".", 1)[0] + f".{os.getpid()}.o")
        if src.endswith(".cpp"):
            cmd = [shutil.which("g++") or "g++", *host_flags, "-c", src, "-o", obj]
        else:
            cmd = [cc, *flags, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed on {os.path.basename(src)}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(one, sources() + host_sources()))
    tmp = LIB + f".{os.getpid()}.tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fopenmp", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    for o in objs:
        try:
            os.remove(o)
        except OSError:
            pass
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
