"""Builds libaf.so (the sm_103a CUDA library) in-tree with nvcc.

Every translation unit compiles in parallel for one target,
``-gencode arch=compute_103a,code=sm_103a``, and links into
``accelerate-fourier_gb300/lib/libaf.so``.  No cmake, no torch extension
machinery: the library is a plain C ABI shared object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG_ROOT, "csrc")
LIBDIR = os.path.join(PKG_ROOT, "lib")
LIB = os.path.join(LIBDIR, "libaf.so")
OBJDIR = os.path.join(PKG_ROOT, "_build")
INCLUDE = os.path.join(os.path.dirname(PKG_ROOT), "include")

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cpp")))


def _headers_mtime() -> float:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "af.h"))
    return max(os.path.getmtime(h) for h in hs)


def _compile(src: str, nvcc: str, hdr_mtime: float) -> str:
    obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
    if src.endswith("64.cu"):
        # the FP64 builds include another translation unit of csrc/
        hdr_mtime = max(hdr_mtime, *(os.path.getmtime(s) for s in sources()))
    if (os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src)
            and os.path.getmtime(obj) >= hdr_mtime):
        return obj
    cmd = [nvcc, *GENCODE, *NVCC_FLAGS, "-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc, *NVCC_FLAGS, "-x", "c++", "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()
    srcs = sources()
    hdr = _headers_mtime()
    if force:
        for f in os.listdir(OBJDIR):
            os.remove(os.path.join(OBJDIR, f))
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, nvcc, hdr), srcs))
    newest = max(os.path.getmtime(o) for o in objs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc, *GENCODE, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print("built", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
