"""Build recipe for libkhronos_gb300.so (sm_103a, in-tree).

The translation units are compiled in parallel with nvcc and linked into
``khronos.jl_gb300/libkhronos_gb300.so``.  No torch extension machinery is
involved: the product is a plain C-ABI shared library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = ROOT / "_build" / "khronos_gb300"
LIB = PKG / "libkhronos_gb300.so"
# Bounds-checked build (-DKH_DEBUG_BOUNDS): every index of the step kernels
# tested against its array's extent, violations recorded for kh_debug_bounds.
BUILD_BOUNDS = ROOT / "_build" / "khronos_gb300_bounds"
LIB_BOUNDS = PKG / "libkhronos_gb300_bounds.so"
SOURCES = ["kh_kernels.cu", "kh_tma.cu", "kh_sim.cu", "kh_serve.cu", "kh_adjoint.cu", "kh_geometry.cu",
           "kh_setup.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# The geometry set-up decides inside/outside at points that can sit exactly on
# an object's boundary: its double arithmetic is kept unfused so each
# coordinate and distance rounds as the IEEE expression it restates.
PER_FILE_FLAGS = {"kh_geometry.cu": ["-fmad=false"]}


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libkhronos_gb300.so")


def _stale(lib: Path = LIB) -> bool:
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    deps = [CSRC / s for s in SOURCES] + [CSRC / h for h in ("kh_kernels.cuh", "kh_cell.cuh", "kh_simbase.h")] + [ROOT / "include" / "khronos_gb300.h"]
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False, bounds: bool = False) -> Path:
    """Compile the library if any source is newer than it; return its path.
    ``bounds`` builds the bounds-checked variant (libkhronos_gb300_bounds.so)."""
    lib, out = (LIB_BOUNDS, BUILD_BOUNDS) if bounds else (LIB, BUILD)
    if not force and not _stale(lib):
        return lib
    out.mkdir(parents=True, exist_ok=True)
    cc = nvcc()
    flags = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2", "-I", str(ROOT / "include")]
    if bounds:
        flags.append("-DKH_DEBUG_BOUNDS")

    def compile_one(src: str) -> Path:
        obj = out / (Path(src).stem + ".o")
        cmd = [cc, *flags, *PER_FILE_FLAGS.get(src, []), "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = lib.with_suffix(".so.tmp")
    cmd = [cc, "-shared", *ARCH, *map(str, objs), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, bounds="--bounds" in sys.argv))
