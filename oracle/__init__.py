"""ORACLE -- test infrastructure only: the CPU restatement of the reference's
FMM GEMM path (fmm_oracle.c), loaded with ctypes. Only tests/, the smoke
check and bench.py's CPU-baseline leg use it, always as the checker or the
timed CPU baseline, never as the product path."""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "fmm_oracle.c"
LIB = HERE / "_build" / "liboracle.so"

_lib = None


def build(force: bool = False) -> Path:
    """gcc -O2 -fopenmp, no FP contraction (the split restatement relies on
    exactly the operations it spells out)."""
    LIB.parent.mkdir(exist_ok=True)
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        tmp = LIB.with_suffix(".tmp.so")
        cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=gnu11",
               str(SRC), "-o", str(tmp), "-lm"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + p.stdout + p.stderr)
        tmp.replace(LIB)
    return LIB


def build_ref() -> bool:
    """Builds the reference itself into oracle/_ref/ (build_ref.sh) where its
    sources are mounted; returns False, doing nothing, where they are not
    (the GPU machine). Only the fixture generator runs what it builds."""
    p = subprocess.run(["bash", str(HERE / "build_ref.sh")], capture_output=True, text=True)
    if p.returncode == 2:
        return False
    if p.returncode != 0:
        raise RuntimeError("reference build failed:\n" + p.stdout[-4000:] + p.stderr[-4000:])
    return True


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB))
        i64, dbl, vp, ci = ctypes.c_int64, ctypes.c_double, ctypes.c_void_p, ctypes.c_int
        ip = ctypes.POINTER(ctypes.c_int)
        L.oracle_fmm_dgemm.restype = ci
        L.oracle_fmm_dgemm.argtypes = [ci, ci, ci, ci, ip, ip, ip, i64, i64, i64, dbl, vp, i64, vp, i64,
                                       dbl, vp, i64, ci, ci]
        L.oracle_split_fmm_dgemm.restype = ci
        L.oracle_split_fmm_dgemm.argtypes = [ci, ci, ci, ci, ip, ip, ip, i64, i64, i64, dbl, vp, i64, vp,
                                             i64, dbl, vp, i64, ci]
        L.oracle_split_fmm_dgemm_fmt.restype = ci
        L.oracle_split_fmm_dgemm_fmt.argtypes = L.oracle_split_fmm_dgemm.argtypes + [ci]
        L.oracle_split_fmm_dgemm_rows.restype = ci
        L.oracle_split_fmm_dgemm_rows.argtypes = L.oracle_split_fmm_dgemm_fmt.argtypes + [vp, i64]
        L.oracle_dgemm.restype = None
        L.oracle_dgemm.argtypes = [i64, i64, i64, dbl, vp, i64, vp, i64, dbl, vp, i64]
        L.oracle_naive_dgemm.restype = None
        L.oracle_naive_dgemm.argtypes = [i64, i64, i64, vp, i64, vp, i64, vp, i64]
        L.oracle_num_threads.restype = ci
        L.oracle_set_threads.restype = None
        L.oracle_set_threads.argtypes = [ci]
        _lib = L
    return _lib


def _f64(x):
    x = np.asarray(x)
    if x.dtype != np.float64 or not x.flags.f_contiguous:
        raise ValueError("oracle arrays must be Fortran-ordered float64")
    return x


def _alg(alg):
    """alg = (mt, kt, nt, R, U, V, W) with U/V/W int32 row-major arrays."""
    mt, kt, nt, R, U, V, W = alg
    U = np.ascontiguousarray(U, dtype=np.int32)
    V = np.ascontiguousarray(V, dtype=np.int32)
    W = np.ascontiguousarray(W, dtype=np.int32)
    ip = ctypes.POINTER(ctypes.c_int)
    return (mt, kt, nt, R, U.ctypes.data_as(ip), V.ctypes.data_as(ip), W.ctypes.data_as(ip)), (U, V, W)


def fmm_dgemm(alg, A, B, C, alpha=1.0, beta=1.0, r_begin=0, r_end=None):
    """C := beta*C + alpha*A*B through the reference algorithm (in place)."""
    A, B, C = _f64(A), _f64(B), _f64(C)
    m, k = A.shape
    n = B.shape[1]
    args, keep = _alg(alg)
    rc = lib().oracle_fmm_dgemm(*args, m, n, k, alpha, A.ctypes.data, max(m, 1), B.ctypes.data, max(k, 1),
                                beta, C.ctypes.data, max(m, 1), r_begin, alg[3] if r_end is None else r_end)
    if rc != 0:
        raise MemoryError("oracle_fmm_dgemm failed")
    return C


def split_fmm_dgemm(alg, A, B, C, slices, alpha=1.0, beta=1.0, fmt="bf16"):
    """The split-precision form's exact arithmetic (in place); fmt "bf16"
    (base-256 digits) or "fp8" (base-32 digits, FP8-E4M3 slices)."""
    A, B, C = _f64(A), _f64(B), _f64(C)
    m, k = A.shape
    n = B.shape[1]
    args, keep = _alg(alg)
    rc = lib().oracle_split_fmm_dgemm_fmt(*args, m, n, k, alpha, A.ctypes.data, max(m, 1), B.ctypes.data,
                                          max(k, 1), beta, C.ctypes.data, max(m, 1), slices,
                                          {"bf16": 0, "fp8": 1}[fmt])
    if rc != 0:
        raise ValueError("oracle_split_fmm_dgemm: unsupported size or allocation failure")
    return C


def split_fmm_dgemm_rows(alg, A, B, C, slices, rows, alpha=1.0, beta=1.0, fmt="bf16"):
    """split_fmm_dgemm restricted to the listed rows i of the product grid
    (0 <= i < ceil(m/m~)): C rows part_offset + i of every C part row get
    exactly the values the full call gives them; other rows get only beta's
    scaling. For checking large problems on a few rows."""
    A, B, C = _f64(A), _f64(B), _f64(C)
    m, k = A.shape
    n = B.shape[1]
    args, keep = _alg(alg)
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    rc = lib().oracle_split_fmm_dgemm_rows(*args, m, n, k, alpha, A.ctypes.data, max(m, 1), B.ctypes.data,
                                           max(k, 1), beta, C.ctypes.data, max(m, 1), slices,
                                           {"bf16": 0, "fp8": 1}[fmt], rows.ctypes.data, len(rows))
    if rc != 0:
        raise ValueError("oracle_split_fmm_dgemm_rows: bad rows, unsupported size or allocation failure")
    return C


def part_rows(d, t, i):
    """Rows (or columns) of a d-long dimension split t ways that local index i
    of the product grid lands on: offset of part p plus i, for every part p
    long enough (frame/base/bli_strassen_ab.c:86-121)."""
    q, r = divmod(d, t)
    out, off = [], 0
    for p in range(t):
        ln = q + (1 if p < r else 0)
        if i < ln:
            out.append(off + i)
        off += ln
    return out


def dgemm(A, B, C, alpha=1.0, beta=1.0):
    A, B, C = _f64(A), _f64(B), _f64(C)
    m, k = A.shape
    n = B.shape[1]
    lib().oracle_dgemm(m, n, k, alpha, A.ctypes.data, max(m, 1), B.ctypes.data, max(k, 1), beta,
                       C.ctypes.data, max(m, 1))
    return C


def naive_dgemm(A, B, C):
    """test/test_strassen_oapi.c:18-42 (C += A*B)."""
    A, B, C = _f64(A), _f64(B), _f64(C)
    m, k = A.shape
    n = B.shape[1]
    lib().oracle_naive_dgemm(m, n, k, A.ctypes.data, max(m, 1), B.ctypes.data, max(k, 1), C.ctypes.data,
                             max(m, 1))
    return C


def set_threads(n: int) -> None:
    lib().oracle_set_threads(n)


def num_threads() -> int:
    return lib().oracle_num_threads()
