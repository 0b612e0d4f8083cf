"""Builds ``_lib/liblightgarden_cuda.so`` for sm_103a with nvcc (no cmake).

``python -m light_garden_gb300.build`` or ``__graft_entry__.build()``.  Translation units
compile in parallel; the shared library links the CUDA runtime statically so it loads
into any process (Python via ctypes, C, C++, Rust via FFI).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIB_DIR = PKG / "_lib"
OBJ_DIR = PKG / "_build"
SOURCES = ["lg_api.cu", "lg_trace.cu", "lg_exact.cu", "lg_raster.cu", "lg_noalloc.cu", "lg_batch.cu", "lg_serve.cu"]
HEADERS = ["lg_device.cuh", "lg_kernels.cuh", "lg_df.cuh", "lg_x64.cuh", "lg_trace_common.cuh", "lg_host.hpp",
           "lg_ctx.hpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False, extra_flags=(), lib_dir: Path = LIB_DIR,
          obj_dir: Path = OBJ_DIR) -> Path:
    """Compile (only what changed) and link the library into ``lib_dir``.  Experiment
    builds pass ``extra_flags`` with their own ``lib_dir`` / ``obj_dir``."""
    lib_dir, obj_dir = Path(lib_dir), Path(obj_dir)
    lib_dir.mkdir(parents=True, exist_ok=True)
    obj_dir.mkdir(parents=True, exist_ok=True)
    headers = [CSRC / h for h in HEADERS] + [PKG.parent / "include" / "lg.h"]
    cc = nvcc()

    def compile_one(src: str) -> Path:
        obj = obj_dir / (Path(src).stem + ".o")
        if force or _stale(obj, [CSRC / src] + headers):
            cmd = [cc, *ARCH, *NVCC_FLAGS, *extra_flags, "-dc", "-o", str(obj), str(CSRC / src)]
            if verbose:
                print(" ".join(cmd), flush=True)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr, flush=True)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    lib = lib_dir / "liblightgarden_cuda.so"
    if force or _stale(lib, objs):
        cmd = [cc, *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-cudart", "static"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    # the benchmark's roofline ceilings (shared-memory atomics, FP32, FP64), measured live
    peaks = lib_dir / "liblg_peaks.so"
    if force or _stale(peaks, [CSRC / "lg_peaks.cu"]):
        cmd = [cc, *ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-o", str(peaks),
               str(CSRC / "lg_peaks.cu"), "-cudart", "static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on lg_peaks.cu:\n{r.stdout}\n{r.stderr}")
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
