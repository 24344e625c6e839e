"""Build libtaufactor_gb300.so in-tree with nvcc for sm_103a (no cmake, no torch extension).

    python -m taufactor_gb300.build            # or __graft_entry__.build()

Each .cu under csrc/ is compiled to an object in parallel, then linked (static cudart) into
taufactor_gb300/lib/libtaufactor_gb300.so. Objects land in taufactor_gb300/_build/.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIBNAME = "libtaufactor_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build taufactor_gb300")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _compile(nvcc, src, verbose_ptxas=False):
    obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
    # -fmad=false: no multiply-add contraction anywhere; every fused operation in the kernels is
    # an explicit fma (the float32 sweeps must round every product and sum on its own).
    cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC", "-c", src, "-o", obj]
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose_ptxas: bool = False, force: bool = False) -> str:
    """Compile and link; returns the library path. Rebuilds when a source is newer."""
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    lib = os.path.join(LIBDIR, LIBNAME)
    srcs = sources()
    deps = srcs + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(os.path.dirname(PKG), "include", "taufactor_gb300.h"))
    if (not force and not verbose_ptxas and os.path.exists(lib)
            and os.path.getmtime(lib) >= max(os.path.getmtime(d) for d in deps)):
        return lib
    nvcc = nvcc_path()
    # one compiler process per translation unit, up to the host's cores (16 on the GPU machines)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(os.cpu_count() or 8, 16, len(srcs)))) as ex:
        results = list(ex.map(lambda s: _compile(nvcc, s, verbose_ptxas), srcs))
    if verbose_ptxas:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = lib + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    path = build(verbose_ptxas="-v" in sys.argv, force="-f" in sys.argv)
    print(path)
