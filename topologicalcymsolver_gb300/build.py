"""In-tree build of the CUDA library (libtcym.so) for sm_103a.

``build_library()`` compiles every translation unit of csrc/ with nvcc in
parallel (objects under ``_build/``) and links ``libtcym.so`` next to this
file; ``build_hostcheck()`` compiles the test-only host instantiation of the
per-site device code (``libtcym_hostcheck.so``).  Rebuilds only when a source
is newer than its output.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libtcym.so")
HOSTCHECK = os.path.join(PKG, "libtcym_hostcheck.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
# translation units of libtcym.so (the host-check unit is built separately)
UNITS = ["tcym_kern_su3_f32.cu", "tcym_kern_su3_f32_batch.cu", "tcym_kern_su3_f64.cu", "tcym_kern_su3_f64_batch.cu",
         "tcym_kern_su2_f32.cu", "tcym_kern_su2_f64.cu", "tcym_reduce.cu", "tcym_capi.cu", "tcym_noalloc.cu",
         "tcym_ensemble.cu", "tcym_serve.cu", "tcym_cooling.cu", "tcym_io.cu", "tcym_autotune.cu", "tcym_snapshot.cu"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtcym.so")


def _sources_mtime() -> float:
    files = glob.glob(os.path.join(CSRC, "*")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files)


def _stale(out: str) -> bool:
    return not os.path.exists(out) or os.path.getmtime(out) < _sources_mtime()


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build_library(force: bool = False, extra: list[str] | None = None) -> str:
    """Compile and link libtcym.so; returns its path."""
    if not force and not _stale(LIB):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    extra = list(extra or [])
    objs = []
    cmds = []
    for u in UNITS:
        obj = os.path.join(BUILD, u.replace(".cu", ".o"))
        objs.append(obj)
        cmds.append([nv, *ARCH, *NVFLAGS, *extra, "-c", os.path.join(CSRC, u), "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        list(ex.map(_run, cmds))
    tmp = LIB + ".tmp"
    _run([nv, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs])
    os.replace(tmp, LIB)
    return LIB


def build_hostcheck(force: bool = False) -> str:
    """Compile the test-only host instantiation of the device site code."""
    if not force and not _stale(HOSTCHECK):
        return HOSTCHECK
    nv = nvcc()
    tmp = HOSTCHECK + ".tmp"
    _run([nv, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr", "-shared",
          os.path.join(CSRC, "tcym_hostcheck.cu"), "-o", tmp])
    os.replace(tmp, HOSTCHECK)
    return HOSTCHECK


if __name__ == "__main__":
    print(build_library(force=True))
    print(build_hostcheck(force=True))
