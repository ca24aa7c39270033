"""Builds the in-tree shared library ``fmm_blis_gb300/libfmm_gb300.so``.

The CUDA translation units are compiled for sm_103a only, in parallel, and
linked with the host C coefficient code into one C-ABI shared library (CUDA
runtime linked statically, so the library loads on machines without a GPU
driver; the driver is only needed once a GPU entry point is called).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libfmm_gb300.so"

CU_SOURCES = ["fmm_api.cu", "fmm_f64.cu", "fmm_split.cu"]
C_SOURCES = ["fmm_coeffs.c"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the fmm_gb300 CUDA library cannot be built")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout + proc.stderr)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compiles (if needed) and returns the path of libfmm_gb300.so."""
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "fmm_gb300.h"]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = CSRC / src
        o = BUILD / (src + ".o")
        objs.append(o)
        if force or _stale(o, [s, *headers]):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-O3", "-c", str(s), "-o", str(o)])
    for src in C_SOURCES:
        s = CSRC / src
        o = BUILD / (src + ".o")
        objs.append(o)
        if force or _stale(o, [s, *headers]):
            jobs.append(["gcc", "-O2", "-fPIC", "-std=c11", "-Wall", "-c", str(s), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    if force or jobs or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "static"])
        os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
