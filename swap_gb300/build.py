"""Build the sm_103a C-ABI library in-tree (swap_gb300/_lib/libswap_gpu.so).

Each translation unit is compiled by nvcc with its own flags, in parallel, and
linked with ``nvcc -shared``.  The FP64 drop-in kernels (k64.cu) are compiled
with ``--fmad=false`` so their rounding follows the Fortran order of
operations; the FP32 form keeps contraction on.  Run ``python -m
swap_gb300.build`` or call :func:`build`.
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
OBJ = PKG / "_build"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libswap_gpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-Xptxas", "-warn-spills"]

# (source, extra flags)
UNITS = [
    ("k64.cu", ["--fmad=false"]),
    ("k32.cu", []),
    ("swap_abi.cu", []),
    ("swap_f32.cu", []),
    ("swap_prof.cu", []),
    ("swap_noalloc.cu", ["--fmad=false"]),
    ("swap_sources.cu", ["--fmad=false", "-Xcompiler", "-ffp-contract=off"]),
    ("loader.cpp", ["-Xcompiler", "-fopenmp,-ffp-contract=off"]),
    ("swap_diag.cu", []),
    ("surrogate.cu", []),
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build swap_gb300")


def _stale(obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile(src: str, flags: list[str], headers: list[Path], verbose: bool) -> Path:
    s = CSRC / src
    o = OBJ / (src + ".o")
    if _stale(o, [s] + headers):
        cmd = [nvcc()] + NVCC_COMMON + flags + ["-x", "cu" if src.endswith(".cu") else "c++", "-c", str(s), "-o", str(o)]
        if src.endswith(".cpp"):
            cmd = [nvcc(), "-O2", "-std=c++17", "-Xcompiler", "-fPIC"] + flags + ["-c", str(s), "-o", str(o)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, flush=True)
    return o


def build(verbose: bool = False) -> Path:
    OBJ.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "swap_gpu.h"]
    units = [(s, f) for s, f in UNITS if (CSRC / s).exists()]
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(lambda u: _compile(u[0], u[1], headers, verbose), units))
    if _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc()] + ARCH + ["-shared", "-Xcompiler", "-fopenmp", "-o", str(tmp)] + [str(o) for o in objs] + ["-lgomp"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
