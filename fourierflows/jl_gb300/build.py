"""Build recipe for libfourierflows_gb300.so (sm_103a), compiled in-tree with nvcc.

Every ``csrc/*.cu`` translation unit is compiled in parallel to an object file under
``csrc/_build/`` and linked into ``libfourierflows_gb300.so`` next to this file.  Objects
are rebuilt when their source or any header is newer.  No torch types cross the
library's C ABI, so the library is plain nvcc + cudart.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(CSRC, "_build")
INCLUDE = os.path.normpath(os.path.join(HERE, "..", "..", "include"))
LIBNAME = "libfourierflows_gb300.so"
LIBPATH = os.path.join(HERE, LIBNAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE,
                     "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfourierflows_gb300")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(obj: str, src: str, hdr_mtime: float) -> bool:
    if not os.path.exists(obj):
        return True
    m = os.path.getmtime(obj)
    return m < os.path.getmtime(src) or m < hdr_mtime


def build_library(verbose: bool = False, force: bool = False, extra_flags=None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdr_mtime = max([os.path.getmtime(h) for h in _headers()] + [0.0])
    flags = NVCC_FLAGS + list(extra_flags or [])
    cc = nvcc()
    jobs = []
    for src in srcs:
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        if force or _stale(obj, src, hdr_mtime):
            jobs.append((src, obj))

    def compile_one(job):
        src, obj = job
        cmd = [cc, "-c", src, "-o", obj] + flags
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, r.returncode, r.stdout + r.stderr

    if jobs:
        workers = min(len(jobs), max(1, os.cpu_count() or 1))
        with cf.ThreadPoolExecutor(workers) as ex:
            for src, rc, out in ex.map(compile_one, jobs):
                if verbose and out.strip():
                    print(out, file=sys.stderr)
                if rc != 0:
                    raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{out}")
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + ".o") for s in srcs]
    if jobs or not os.path.exists(LIBPATH) or any(os.path.getmtime(o) > os.path.getmtime(LIBPATH) for o in objs):
        tmp = LIBPATH + ".tmp"
        cmd = [cc, "-shared", "-o", tmp] + objs + ARCH + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}{r.stderr}")
        os.replace(tmp, LIBPATH)
    return LIBPATH


if __name__ == "__main__":
    print(build_library(verbose=True, force="--force" in sys.argv))
