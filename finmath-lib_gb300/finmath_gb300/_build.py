"""Build of the native library liblmm_gb300.so (CUDA kernels for sm_103a + C ABI).

nvcc compiles each .cu translation unit for sm_103a only; the FP64 parity units are
compiled with -fmad=false so that every add and multiply rounds separately, as the
reference's Java arithmetic does.  Host C++ is compiled with -ffp-contract=off for the
same reason.  Objects are built in parallel and linked with the static CUDA runtime.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)                    # finmath-lib_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(BUILD, "liblmm_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# translation units whose FP64 arithmetic must not be contracted into FMAs
NO_FMAD = {"rng.cu", "paths_fp64.cu", "paths_fp64_n64.cu", "paths_fp64_n80.cu", "products.cu", "randomvariable.cu"}


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _deps_mtime() -> float:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return max(os.path.getmtime(f) for f in files)


def _compile(src: str, nvcc: str) -> str:
    obj = os.path.join(BUILD, src + ".o")
    path = os.path.join(CSRC, src)
    if src.endswith(".cu"):
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
               "-I", INCLUDE, "-I", CSRC, "-c", path, "-o", obj]
        if src in NO_FMAD:
            cmd.insert(1, "-fmad=false")
        if os.environ.get("LMM_PTXAS_VERBOSE"):
            cmd += ["-Xptxas", "-v"]
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC,
               "-I", os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include"), "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if os.environ.get("LMM_PTXAS_VERBOSE"):
        print(r.stderr)
    return obj


def build(force: bool = False) -> str:
    """Compile and link liblmm_gb300.so in-tree; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    nvcc = _nvcc()
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, nvcc), srcs))
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static", "-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
