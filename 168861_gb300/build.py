"""Builds libneurite_gb300.so (the CUDA extension) in-tree with nvcc for sm_103a.

Translation units compile in parallel, then link into 168861_gb300/_build/.  The
library is plain C ABI (include/neurite_gb300.h); Python loads it with ctypes.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libneurite_gb300.so")
SOURCES = ["api.cu", "explicit.cu", "implicit.cu", "derive.cpp", "serve.cpp", "static_solve.cu", "record.cu", "derive_device.cu", "strain.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags(extra=()):
    return ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", CSRC, "-I",
            os.path.join(ROOT, "include"), *ARCH, *extra]


def _needs(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "neurite_gb300.h"))
    cc = nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OUT, src.rsplit(".", 1)[0] + ".o")
        objs.append(obj)
        if force or _needs(obj, [path, *headers]):
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            lang = ["-x", "cu"] if src.endswith(".cu") else []
            jobs.append([cc, *_flags(extra), *lang, "-c", path, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose or ptxas_info:
            sys.stderr.write(r.stderr)
        return r

    with cf.ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        run([cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-Xcompiler", "-pthread"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv))
