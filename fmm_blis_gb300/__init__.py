"""Python mirror of the fmm-blis FMM GEMM interface over the GB300 C ABI.

The compute path is the CUDA library ``libfmm_gb300.so`` (include/fmm_gb300.h);
this module only loads it with ctypes and converts arguments. There is no
CPU fallback: if the library is missing, ``lib()`` raises.

Names follow the reference's interface (frame/include/bli_fmm.h:61-89):
``new_fmm``/``free_fmm`` read and release a coefficient algorithm,
``STRASSEN_FMM`` is the built-in Strassen <2,2,2>, ``bli_strassen_ab_ex``
computes C += A*B through one FMM level (host arrays, like the reference's
obj_t call), ``bl_clock`` is the monotonic timer. The device-resident forms are
``dgemm`` (plain FP64) and ``split_dgemm`` (BF16 digit slices on the tensor
cores), both taking column-major CUDA tensors.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libfmm_gb300.so"

FMM_OK = 0
_STATUS = {
    0: "ok", 1: "invalid argument", 2: "coefficient file cannot be opened",
    3: "coefficient file malformed", 4: "allocation failed", 5: "CUDA call failed",
    6: "unsupported size or option", 7: "coefficients violate the Brent equations",
    8: "kernel reported an error (bounded wait expired)", 9: "workspace too small",
    10: "problem larger than the static scratch of the allocation-free entry point",
}


class FmmError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        super().__init__(f"{what}: {_STATUS.get(status, 'unknown status')} (status {status})")


class BatchProblem(ctypes.Structure):
    """fmm_batch_problem (include/fmm_gb300.h)."""

    _fields_ = [
        ("fmm", ctypes.c_void_p), ("levels", ctypes.c_int), ("slices", ctypes.c_int),
        ("m", ctypes.c_int64), ("n", ctypes.c_int64), ("k", ctypes.c_int64),
        ("alpha", ctypes.c_double), ("A", ctypes.c_void_p), ("lda", ctypes.c_int64),
        ("B", ctypes.c_void_p), ("ldb", ctypes.c_int64),
        ("beta", ctypes.c_double), ("C", ctypes.c_void_p), ("ldc", ctypes.c_int64),
        ("format", ctypes.c_int),
    ]


class FmmT(ctypes.Structure):
    """Same layout as the reference's fmm_t (plugin/bli_plugin_fmm_blis.h:58-68)."""

    _fields_ = [
        ("m_tilde", ctypes.c_int),
        ("n_tilde", ctypes.c_int),
        ("k_tilde", ctypes.c_int),
        ("R", ctypes.c_int),
        ("U", ctypes.POINTER(ctypes.c_int)),
        ("V", ctypes.POINTER(ctypes.c_int)),
        ("W", ctypes.POINTER(ctypes.c_int)),
    ]

    def coeffs(self):
        """(U, V, W) as lists of rows (row q, column r)."""
        R = self.R
        a = self.m_tilde * self.k_tilde
        b = self.k_tilde * self.n_tilde
        c = self.m_tilde * self.n_tilde
        U = [[self.U[q * R + r] for r in range(R)] for q in range(a)]
        V = [[self.V[q * R + r] for r in range(R)] for q in range(b)]
        W = [[self.W[q * R + r] for r in range(R)] for q in range(c)]
        return U, V, W


_lib = None


def lib() -> ctypes.CDLL:
    """The loaded CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build it with fmm_blis_gb300.build.build()")
    L = ctypes.CDLL(str(LIB_PATH))
    i64, dbl, vp, ci = ctypes.c_int64, ctypes.c_double, ctypes.c_void_p, ctypes.c_int
    pf = ctypes.POINTER(FmmT)
    L.new_fmm.restype = FmmT
    L.new_fmm.argtypes = [ctypes.c_char_p]
    L.free_fmm.restype = None
    L.free_fmm.argtypes = [FmmT]
    L.fmm_load.restype = ci
    L.fmm_load.argtypes = [ctypes.c_char_p, pf]
    L.fmm_check_brent.restype = ci
    L.fmm_check_brent.argtypes = [pf, ctypes.POINTER(ctypes.c_long)]
    L.fmm_kron.restype = ci
    L.fmm_kron.argtypes = [pf, pf, pf]
    L.fmm_copy.restype = ci
    L.fmm_copy.argtypes = [pf, pf]
    L.fmm_status_string.restype = ctypes.c_char_p
    L.fmm_status_string.argtypes = [ci]
    L.bl_clock.restype = dbl
    L.bl_clock.argtypes = []
    L.fmm_gpu_dgemm.restype = ci
    L.fmm_gpu_dgemm.argtypes = [pf, ci, i64, i64, i64, dbl, vp, i64, vp, i64, dbl, vp, i64, vp]
    L.fmm_gpu_strassen_ab_ex.restype = ci
    L.fmm_gpu_strassen_ab_ex.argtypes = [dbl, vp, i64, vp, i64, dbl, vp, i64, i64, i64, i64, FmmT]
    L.fmm_gpu_strassen_ab_gen.restype = ci
    L.fmm_gpu_strassen_ab_gen.argtypes = [dbl, vp, i64, i64, vp, i64, i64, dbl, vp, i64, i64, i64, i64, i64, FmmT]
    L.fmm_gpu_split_strassen_ab_ex.restype = ci
    L.fmm_gpu_split_strassen_ab_ex.argtypes = [dbl, vp, i64, vp, i64, dbl, vp, i64, i64, i64, i64, FmmT, ci, ci, ci]
    L.fmm_gpu_split_strassen_ab_gen.restype = ci
    L.fmm_gpu_split_strassen_ab_gen.argtypes = [dbl, vp, i64, i64, vp, i64, i64, dbl, vp, i64, i64, i64, i64, i64,
                                                FmmT, ci, ci, ci]
    L.fmm_gpu_release_host_buffers.restype = None
    L.fmm_gpu_release_host_buffers.argtypes = []
    L.fmm_gpu_host_alloc.restype = ci
    L.fmm_gpu_host_alloc.argtypes = [ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]
    L.fmm_gpu_host_free.restype = ci
    L.fmm_gpu_host_free.argtypes = [ctypes.c_void_p]
    L.fmm_gpu_strassen_ab.restype = ci
    L.fmm_gpu_strassen_ab.argtypes = [dbl, vp, i64, vp, i64, dbl, vp, i64, i64, i64, i64]
    L.fmm_gpu_split_workspace_size.restype = ctypes.c_size_t
    L.fmm_gpu_split_workspace_size.argtypes = [pf, ci, i64, i64, i64, ci]
    L.fmm_gpu_split_workspace_size_fmt.restype = ctypes.c_size_t
    L.fmm_gpu_split_workspace_size_fmt.argtypes = [pf, ci, i64, i64, i64, ci, ci]
    L.fmm_gpu_split_dgemm_fmt.restype = ci
    L.fmm_gpu_split_dgemm_fmt.argtypes = [pf, ci, i64, i64, i64, dbl, vp, i64, vp, i64, dbl, vp, i64, ci, ci, vp,
                                          ctypes.c_size_t, vp]
    L.fmm_gpu_split_dgemm.restype = ci
    L.fmm_gpu_split_dgemm.argtypes = [pf, ci, i64, i64, i64, dbl, vp, i64, vp, i64, dbl, vp, i64, ci, vp,
                                      ctypes.c_size_t, vp]
    L.fmm_gpu_batch_workspace_size.restype = ctypes.c_size_t
    L.fmm_gpu_batch_workspace_size.argtypes = [ci, ctypes.POINTER(BatchProblem)]
    L.fmm_gpu_batch_dgemm.restype = ci
    L.fmm_gpu_batch_dgemm.argtypes = [ci, ctypes.POINTER(BatchProblem), vp, ctypes.c_size_t, vp]
    L.fmm_gpu_selftest_wait_expiry.restype = ci
    L.fmm_gpu_selftest_wait_expiry.argtypes = [ctypes.POINTER(ci)]
    L.fmm_gpu_set_f64_batch_ctas.restype = ci
    L.fmm_gpu_set_f64_batch_ctas.argtypes = [ci]
    L.fmm_gpu_set_f64_engine.restype = ci
    L.fmm_gpu_set_f64_engine.argtypes = [ci]
    L.fmm_gpu_f64_sup_splits.restype = ci
    L.fmm_gpu_f64_sup_splits.argtypes = [i64, i64, i64]
    L.fmm_gpu_set_host_timeline.restype = None
    L.fmm_gpu_set_host_timeline.argtypes = [ci]
    L.fmm_gpu_read_host_timeline.restype = ci
    L.fmm_gpu_read_host_timeline.argtypes = [ctypes.POINTER(dbl), ci]
    L.fmm_gpu_fp64_pipe_rates.restype = ci
    L.fmm_gpu_fp64_pipe_rates.argtypes = [ctypes.POINTER(dbl), ctypes.POINTER(dbl), ctypes.POINTER(dbl)]
    L.fmm_gpu_split_dgemm_noalloc.restype = ci
    L.fmm_gpu_split_dgemm_noalloc.argtypes = [pf, ci, i64, i64, i64, dbl, vp, i64, vp, i64, dbl, vp, i64, ci, vp]
    L.fmm_gpu_set_kernel_timing.restype = None
    L.fmm_gpu_set_kernel_timing.argtypes = [ci]
    L.fmm_gpu_read_kernel_timing.restype = ci
    L.fmm_gpu_read_kernel_timing.argtypes = [ctypes.POINTER(dbl), ctypes.POINTER(ctypes.c_uint64),
                                             ctypes.POINTER(ctypes.c_uint64)]
    L.fmm_gpu_launch_count.restype = ctypes.c_uint64
    L.fmm_gpu_launch_count.argtypes = []
    L.fmm_gpu_take_device_error.restype = ci
    L.fmm_gpu_take_device_error.argtypes = []
    L.fmm_gpu_set_split_pair_rows.restype = ci
    L.fmm_gpu_set_split_pair_rows.argtypes = [ci]
    _lib = L
    return L


def _check(status: int, what: str) -> None:
    if status != FMM_OK:
        raise FmmError(status, what)


# ------------------------------------------------------------ algorithms --

def new_fmm(path: str | os.PathLike) -> FmmT:
    """Reads a coefficient file (frame/base/bli_read_fmm.c:24-80); raises on error."""
    f = FmmT()
    _check(lib().fmm_load(str(path).encode(), ctypes.byref(f)), f"new_fmm({path})")
    return f


def free_fmm(f: FmmT) -> None:
    """Releases an algorithm from new_fmm/kron (frame/base/bli_read_fmm.c:82-86)."""
    lib().free_fmm(f)


def strassen_fmm() -> FmmT:
    """The built-in Strassen <2,2,2> algorithm (frame/base/bli_strassen_ab.c:12-24)."""
    return FmmT.in_dll(lib(), "STRASSEN_FMM")


def check_brent(f: FmmT) -> int:
    """Number of violated Brent equations (0 for a correct algorithm)."""
    bad = ctypes.c_long(0)
    lib().fmm_check_brent(ctypes.byref(f), ctypes.byref(bad))
    return bad.value


def kron(outer: FmmT, inner: FmmT) -> FmmT:
    """Two levels as one flat algorithm (free with free_fmm)."""
    out = FmmT()
    _check(lib().fmm_kron(ctypes.byref(outer), ctypes.byref(inner), ctypes.byref(out)), "fmm_kron")
    return out


def bl_clock() -> float:
    return lib().bl_clock()


def launch_count() -> int:
    """Kernels this library has launched since it was loaded."""
    return int(lib().fmm_gpu_launch_count())


def set_kernel_timing(enable: bool) -> None:
    """Record CUDA events around each split GEMM kernel launch."""
    lib().fmm_gpu_set_kernel_timing(1 if enable else 0)


def read_kernel_timing() -> tuple[float, int, int]:
    """(total milliseconds, launches, products computed) of the timed GEMM
    launches since the last read."""
    ms = ctypes.c_double(0.0)
    n = ctypes.c_uint64(0)
    p = ctypes.c_uint64(0)
    _check(lib().fmm_gpu_read_kernel_timing(ctypes.byref(ms), ctypes.byref(n), ctypes.byref(p)),
           "read_kernel_timing")
    return ms.value, int(n.value), int(p.value)


F64_ENGINES = {"dfma": 0, "mma": 1}


def f64_sup_splits(m: int, n: int, k: int) -> int:
    """k chunks the plain FP64 form's small/skinny classical path uses for an
    m x n x k classical problem (0: the regular kernel); host-only."""
    return int(lib().fmm_gpu_f64_sup_splits(m, n, k))


def set_f64_engine(engine: str) -> str:
    """Micro-kernel of the plain FP64 form: "dfma" or "mma" (FP64 tensor-core
    mma.sync); returns the previous one."""
    prev = lib().fmm_gpu_set_f64_engine(F64_ENGINES[engine])
    if prev < 0:
        raise ValueError(engine)
    return {v: k for k, v in F64_ENGINES.items()}[prev]


def fp64_pipe_rates() -> tuple[float, float, float]:
    """(DFMA, FP64 MMA, both interleaved) peak TFLOP/s measured on the
    current GPU."""
    a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    _check(lib().fmm_gpu_fp64_pipe_rates(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)), "fmm_gpu_fp64_pipe_rates")
    return a.value, b.value, c.value


def selftest_wait_expiry() -> tuple[int, int]:
    """Runs the bounded-wait failure path on purpose (a wait nothing
    completes); returns (status, threads that gave up): (FMM_ERR_DEVICE, 64)
    when it worked."""
    g = ctypes.c_int()
    st = lib().fmm_gpu_selftest_wait_expiry(ctypes.byref(g))
    return st, g.value


def take_device_error() -> int:
    return int(lib().fmm_gpu_take_device_error())


def set_f64_batch_ctas(max_ctas: int) -> int:
    """Caps the CTAs of the FP64 batch launch (0: two per SM); returns the
    previous cap."""
    return lib().fmm_gpu_set_f64_batch_ctas(int(max_ctas))


def set_split_pair_rows(min_rows: int) -> int:
    """Per-product row count m_e from which split GEMMs use CTA-pair tiles
    (default 1024; a huge value keeps single-SM tiles). Same bits either
    way. Returns the previous value."""
    return int(lib().fmm_gpu_set_split_pair_rows(min(int(min_rows), 2**31 - 1)))


# ------------------------------------------------------------ GPU calls --

def _colmajor_ld(t, rows: int, name: str) -> int:
    if t.dtype.__str__() != "torch.float64":
        raise TypeError(f"{name} must be float64")
    if not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dim() != 2:
        raise ValueError(f"{name} must be a 2-D tensor")
    if t.numel() == 0:
        return max(rows, 1)
    if t.shape[0] > 1 and t.stride(0) != 1:
        raise ValueError(f"{name} must be a column-major 2-D tensor (stride(0) == 1)")
    return max(int(t.stride(1)), max(rows, 1))


def colmajor(t):
    """A column-major (Fortran-order) copy/view of a 2-D torch tensor."""
    return t.t().contiguous().t()


def _stream_ptr(stream) -> int | None:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return int(getattr(stream, "cuda_stream", stream))


def dgemm(A, B, C, fmm: FmmT | None = None, levels: int = 1, alpha: float = 1.0, beta: float = 1.0,
          stream=None) -> None:
    """C := beta*C + alpha*A*B on the GPU in FP64 with `levels` levels of `fmm`
    (fmm None or levels 0: the classical FP64 kernel). Column-major tensors."""
    m, k = A.shape
    k2, n = B.shape
    if k2 != k or tuple(C.shape) != (m, n):
        raise ValueError("shape mismatch")
    lda, ldb, ldc = _colmajor_ld(A, m, "A"), _colmajor_ld(B, k, "B"), _colmajor_ld(C, m, "C")
    pf = ctypes.byref(fmm) if fmm is not None else None
    st = lib().fmm_gpu_dgemm(pf, levels if fmm is not None else 0, m, n, k, alpha, A.data_ptr(), lda,
                             B.data_ptr(), ldb, beta, C.data_ptr(), ldc, _stream_ptr(stream))
    _check(st, "fmm_gpu_dgemm")


SPLIT_FORMATS = {"bf16": 0, "fp8": 1}   # FMM_SPLIT_BF16, FMM_SPLIT_FP8_E4M3


def _fmt(fmt) -> int:
    if isinstance(fmt, str):
        if fmt not in SPLIT_FORMATS:
            raise ValueError(f"unknown slice format {fmt!r}")
        return SPLIT_FORMATS[fmt]
    return int(fmt)


def split_workspace_size(m: int, n: int, k: int, fmm: FmmT | None, levels: int, slices: int, fmt="bf16") -> int:
    pf = ctypes.byref(fmm) if fmm is not None else None
    return int(lib().fmm_gpu_split_workspace_size_fmt(pf, levels if fmm is not None else 0, m, n, k, slices,
                                                      _fmt(fmt)))


def split_dgemm(A, B, C, fmm: FmmT | None = None, levels: int = 1, slices: int = 6, alpha: float = 1.0,
                beta: float = 1.0, workspace=None, stream=None, fmt="bf16") -> None:
    """C := beta*C + alpha*A*B from digit slices on the tensor cores: fmt
    "bf16" (8-bit digits, slices 2..8) or "fp8" (5-bit digits as FP8-E4M3,
    slices 2..12). `workspace` is a CUDA uint8 tensor of at least
    split_workspace_size bytes (allocated here when None)."""
    import torch
    m, k = A.shape
    k2, n = B.shape
    if k2 != k or tuple(C.shape) != (m, n):
        raise ValueError("shape mismatch")
    lda, ldb, ldc = _colmajor_ld(A, m, "A"), _colmajor_ld(B, k, "B"), _colmajor_ld(C, m, "C")
    need = split_workspace_size(m, n, k, fmm, levels, slices, fmt)
    if workspace is None:
        workspace = torch.empty(max(need, 256), dtype=torch.uint8, device=C.device)
    pf = ctypes.byref(fmm) if fmm is not None else None
    st = lib().fmm_gpu_split_dgemm_fmt(pf, levels if fmm is not None else 0, m, n, k, alpha, A.data_ptr(), lda,
                                       B.data_ptr(), ldb, beta, C.data_ptr(), ldc, slices, _fmt(fmt),
                                       workspace.data_ptr(), workspace.numel(), _stream_ptr(stream))
    _check(st, "fmm_gpu_split_dgemm")


def split_dgemm_noalloc(A, B, C, fmm: FmmT | None = None, levels: int = 1, slices: int = 6,
                        alpha: float = 1.0, beta: float = 1.0, stream=None) -> None:
    """split_dgemm without any device allocation: the workspace is the
    library's static 64 MiB device scratch (FmmError status 10 when the
    problem does not fit). Calls that overlap on the GPU race on the scratch."""
    m, k = A.shape
    k2, n = B.shape
    if k2 != k or tuple(C.shape) != (m, n):
        raise ValueError("shape mismatch")
    lda, ldb, ldc = _colmajor_ld(A, m, "A"), _colmajor_ld(B, k, "B"), _colmajor_ld(C, m, "C")
    pf = ctypes.byref(fmm) if fmm is not None else None
    st = lib().fmm_gpu_split_dgemm_noalloc(pf, levels if fmm is not None else 0, m, n, k, alpha, A.data_ptr(),
                                           lda, B.data_ptr(), ldb, beta, C.data_ptr(), ldc, slices,
                                           _stream_ptr(stream))
    _check(st, "fmm_gpu_split_dgemm_noalloc")


def make_batch(problems):
    """problems: iterable of dicts with keys A, B, C (column-major CUDA
    tensors), and optional fmm (FmmT or None), levels, slices (0: plain FP64
    form), fmt ("bf16" or "fp8" slices), alpha, beta. Returns a ctypes array
    of fmm_batch_problem."""
    probs = list(problems)
    arr = (BatchProblem * max(len(probs), 1))()
    for i, p in enumerate(probs):
        A, B, C = p["A"], p["B"], p["C"]
        m, k = A.shape
        n = B.shape[1]
        f = p.get("fmm")
        arr[i].fmm = ctypes.cast(ctypes.pointer(f), ctypes.c_void_p) if f is not None else None
        arr[i].levels = p.get("levels", 1) if f is not None else 0
        arr[i].slices = p.get("slices", 6)
        arr[i].m, arr[i].n, arr[i].k = m, n, k
        arr[i].alpha, arr[i].beta = p.get("alpha", 1.0), p.get("beta", 1.0)
        arr[i].A, arr[i].lda = A.data_ptr(), _colmajor_ld(A, m, "A")
        arr[i].B, arr[i].ldb = B.data_ptr(), _colmajor_ld(B, k, "B")
        arr[i].C, arr[i].ldc = C.data_ptr(), _colmajor_ld(C, m, "C")
        arr[i].format = _fmt(p.get("fmt", "bf16"))
    return arr, len(probs)


def batch_workspace_size(batch) -> int:
    arr, count = batch
    return int(lib().fmm_gpu_batch_workspace_size(count, arr))


def batch_shapes_workspace_size(shapes) -> int:
    """Workspace a batch needs, from its problems' shapes and plans alone:
    shapes is an iterable of (m, n, k, fmm or None, levels, slices, fmt). The
    sizing call reads no operand data, so placeholder addresses stand in for
    the operands."""
    items = list(shapes)
    arr = (BatchProblem * max(len(items), 1))()
    for i, (m, n, k, fmm, levels, slices, fmt) in enumerate(items):
        arr[i].fmm = ctypes.cast(ctypes.pointer(fmm), ctypes.c_void_p) if fmm is not None else None
        arr[i].levels = levels if fmm is not None else 0
        arr[i].slices = slices
        arr[i].m, arr[i].n, arr[i].k = m, n, k
        arr[i].alpha, arr[i].beta = 1.0, 1.0
        arr[i].A, arr[i].lda = 256, max(m, 1)
        arr[i].B, arr[i].ldb = 256, max(k, 1)
        arr[i].C, arr[i].ldc = 256, max(m, 1)
        arr[i].format = _fmt(fmt)
    return int(lib().fmm_gpu_batch_workspace_size(len(items), arr))


def batch_problem_workspace_size(m: int, n: int, k: int, fmm: FmmT | None, levels: int, slices: int,
                                 fmt="bf16") -> int:
    """Workspace one problem of this shape needs inside a batch (all of its
    products at once), from the shape alone."""
    return batch_shapes_workspace_size([(m, n, k, fmm, levels, slices, fmt)])


def batch_dgemm(problems, workspace=None, stream=None) -> None:
    """Runs independent GEMMs as one batch (see fmm_gpu_batch_dgemm)."""
    import torch
    arr, count = make_batch(problems) if not isinstance(problems, tuple) else problems
    if count == 0:
        return
    if workspace is None:
        need = int(lib().fmm_gpu_batch_workspace_size(count, arr))
        workspace = torch.empty(max(need, 256), dtype=torch.uint8, device="cuda")
    _check(lib().fmm_gpu_batch_dgemm(count, arr, workspace.data_ptr(), workspace.numel(), _stream_ptr(stream)),
           "fmm_gpu_batch_dgemm")


def split_strassen_ab_ex(alpha: float, A, B, beta: float, C, fmm: FmmT | None = None, levels: int = 1,
                         slices: int = 6, fmt: str = "bf16") -> None:
    """The split form on host arrays: numpy float64 arrays of any layout
    (Fortran order, C order, transposed or strided views) or column-major CPU
    tensors (pinned copies fastest). C updated in place, synchronously; with
    column-major operands the host<->device copies overlap the device work."""
    import numpy as np

    arrays = [x for x in (A, B, C) if isinstance(x, np.ndarray)]
    if len(arrays) == 3 and not all(x.flags.f_contiguous or x.size == 0 for x in arrays):
        for name, x in (("A", A), ("B", B), ("C", C)):
            if x.dtype != np.float64 or x.ndim != 2:
                raise ValueError(f"{name} must be a 2-D float64 array")
            if x.size > 0 and any(st <= 0 or st % 8 for st in x.strides):
                raise ValueError(f"{name} needs positive element strides")
        m, k = A.shape
        n = B.shape[1]
        if B.shape[0] != k or C.shape != (m, n):
            raise ValueError("shape mismatch")

        def rs(x):
            return max(x.strides[0] // 8, 1)

        def cs(x):
            return max(x.strides[1] // 8, 1)

        st = lib().fmm_gpu_split_strassen_ab_gen(alpha, A.ctypes.data, rs(A), cs(A), B.ctypes.data, rs(B), cs(B),
                                                 beta, C.ctypes.data, rs(C), cs(C), m, n, k,
                                                 fmm if fmm is not None else FmmT(),
                                                 levels if fmm is not None else 0, slices, _fmt(fmt))
        _check(st, "fmm_gpu_split_strassen_ab_gen")
        return

    def info(x, name):
        if isinstance(x, np.ndarray):
            if x.dtype != np.float64 or x.ndim != 2 or not (x.flags.f_contiguous or x.size == 0):
                raise ValueError(f"{name} must be a 2-D Fortran-order float64 array")
            return x.ctypes.data, x.shape
        if getattr(x, "is_cuda", True) or str(x.dtype) != "torch.float64" or x.dim() != 2:
            raise ValueError(f"{name} must be a 2-D float64 host array or CPU tensor")
        if x.numel() > 0 and (x.stride(0) != 1 or x.stride(1) < max(x.shape[0], 1)):
            raise ValueError(f"{name} must be column-major")
        return x.data_ptr(), tuple(x.shape)

    pa, (m, k) = info(A, "A")
    pb, (kb, n) = info(B, "B")
    pc, sc = info(C, "C")
    if kb != k or sc != (m, n):
        raise ValueError("shape mismatch")
    st = lib().fmm_gpu_split_strassen_ab_ex(alpha, pa, max(m, 1), pb, max(k, 1), beta, pc, max(m, 1), m, n, k,
                                            fmm if fmm is not None else FmmT(), levels if fmm is not None else 0,
                                            slices, _fmt(fmt))
    _check(st, "fmm_gpu_split_strassen_ab_ex")


HOST_TIMELINE = ("a_up", "b_up", "gemm_start", "gemm_end", "c_down", "host_wall")


def set_host_timeline(enable: bool) -> None:
    lib().fmm_gpu_set_host_timeline(1 if enable else 0)


def read_host_timeline() -> dict:
    """The last host-buffer split call's timeline in milliseconds (see
    fmm_gpu_read_host_timeline)."""
    buf = (ctypes.c_double * len(HOST_TIMELINE))()
    c = lib().fmm_gpu_read_host_timeline(buf, len(HOST_TIMELINE))
    return {k: buf[x] for x, k in enumerate(HOST_TIMELINE[:c])}


def release_host_buffers() -> None:
    """Frees the device buffers kept by split_strassen_ab_ex on this device."""
    lib().fmm_gpu_release_host_buffers()


def host_empty(rows: int, cols: int):
    """A zeroed Fortran-order float64 numpy array of rows x cols in pinned
    host memory on huge pages (fmm_gpu_host_alloc), for the operands of the
    host-buffer calls; freed when the array (and every view of it, e.g.
    torch.from_numpy) is gone. Needs a GPU."""
    import weakref

    import numpy as np

    nbytes = max(rows * cols * 8, 8)
    p = ctypes.c_void_p()
    _check(lib().fmm_gpu_host_alloc(nbytes, ctypes.byref(p)), "fmm_gpu_host_alloc")
    buf = (ctypes.c_double * max(rows * cols, 1)).from_address(p.value)
    arr = np.ctypeslib.as_array(buf)[: rows * cols].reshape((rows, cols), order="F")
    weakref.finalize(arr, lib().fmm_gpu_host_free, p.value)
    return arr


def bli_strassen_ab_ex(alpha: float, A, B, beta: float, C, fmm: FmmT) -> None:
    """Host-array drop-in for bli_strassen_ab_ex (frame/base/bli_strassen_ab.c:123):
    numpy float64 arrays of any layout (Fortran order, C order, transposed or
    strided views, like the obj_t operands of the reference), C updated in
    place."""
    import numpy as np
    for name, x in (("A", A), ("B", B), ("C", C)):
        if x.dtype != np.float64 or x.ndim != 2:
            raise ValueError(f"{name} must be a 2-D float64 array")
        if x.size > 0 and any(st <= 0 or st % 8 for st in x.strides):
            raise ValueError(f"{name} needs positive element strides")
    m, k = A.shape
    n = B.shape[1]
    if B.shape[0] != k or C.shape != (m, n):
        raise ValueError("shape mismatch")
    if A.flags.f_contiguous and B.flags.f_contiguous and C.flags.f_contiguous:
        st = lib().fmm_gpu_strassen_ab_ex(alpha, A.ctypes.data, max(m, 1), B.ctypes.data, max(k, 1), beta,
                                          C.ctypes.data, max(m, 1), m, n, k, fmm)
        _check(st, "fmm_gpu_strassen_ab_ex")
        return

    def rs(x):
        return max(x.strides[0] // 8, 1)

    def cs(x):
        return max(x.strides[1] // 8, 1)

    st = lib().fmm_gpu_strassen_ab_gen(alpha, A.ctypes.data, rs(A), cs(A), B.ctypes.data, rs(B), cs(B), beta,
                                       C.ctypes.data, rs(C), cs(C), m, n, k, fmm)
    _check(st, "fmm_gpu_strassen_ab_gen")
