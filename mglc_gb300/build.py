"""Build libmglc_gb300.so in-tree with nvcc for sm_103a (GB300).

Each .cu under csrc/ compiles to an object in parallel; the objects link into
``mglc_gb300/_build/libmglc_gb300.so``.  No cmake, no torch extension
machinery: the library is a plain C-ABI shared object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
# MGLC_BOUNDS_CHECK=1: the diagnostic build whose step kernels check every
# element index (counted, access skipped), in a directory of its own
CHECKED = os.environ.get("MGLC_BOUNDS_CHECK") == "1"
BUILD = os.path.join(HERE, "_build_checked" if CHECKED else "_build")
LIB = os.path.join(BUILD, "libmglc_gb300.so")
ROOF_LIB = os.path.join(BUILD, "libmglc_roof.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no multiply-add contraction, so host-side constants (relaxation
# rates, sums) round the same on x86-64 and aarch64 hosts
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fno-strict-aliasing", "-Xcompiler", "-ffp-contract=off",
              "-I" + os.path.join(HERE, "..", "include")] + (["-DMGLC_BOUNDS_CHECK"] if CHECKED else [])


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmglc_gb300")
    return p


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "mglc.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


# per-file flags: the 2-D particle and 2-D lid steps reproduce the reference's
# FP64 statements, so no device multiply-add contraction there
FILE_FLAGS = {"k_particle2d.cu": ["-fmad=false"], "k_lid2d.cu": ["-fmad=false"]}


def _compile(src, verbose_ptxas=False):
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
    if not _stale(obj, src):
        return obj, ""
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *FILE_FLAGS.get(os.path.basename(src), []), "-c", src, "-o", obj]
    if verbose_ptxas:
        cmd[1:1] = ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    objs = [o for o, _ in results]
    if verbose_ptxas:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    build_roof()
    return LIB


def build_roof() -> str:
    """The FP64 instruction-rate probe (measurement only, its own library)."""
    src = os.path.join(HERE, "roof", "fp64_rate.cu")
    if os.path.exists(ROOF_LIB) and os.path.getmtime(ROOF_LIB) >= os.path.getmtime(src):
        return ROOF_LIB
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
           src, "-o", ROOF_LIB, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return ROOF_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
