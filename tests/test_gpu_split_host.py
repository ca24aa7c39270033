"""The split form on host buffers (fmm_gpu_split_strassen_ab_ex): operands in
host memory, copies overlapped with the device work inside the call. Every
result equals the device-pointer call's (fmm_gpu_split_dgemm_fmt) bit for bit
and, at sizes the oracle finishes, the oracle's restatement."""
import numpy as np
import pytest

from conftest import COEFFS, rand
from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def device_call(fmm, f, levels, A, B, C, s, fmt, alpha=1.0, beta=1.0):
    dC = to_dev(C)
    fmm.split_dgemm(to_dev(A), to_dev(B), dC, f, levels, s, fmt=fmt, alpha=alpha, beta=beta)
    return to_host(dC)


@pytest.mark.parametrize("fmt,s", [("bf16", 6), ("fp8", 9)])
@pytest.mark.parametrize("shape", [(1, 1, 1), (65, 70, 33), (300, 129, 260)])
def test_host_call_matches_oracle(fmm, orc, algs, torch_cuda, fmt, s, shape):
    m, n, k = shape
    A, B, C = rand(m, k, 501), rand(k, n, 502), rand(m, n, 503)
    got = C.copy(order="F")
    fmm.split_strassen_ab_ex(0.5, A, B, -1.25, got, fmm.strassen_fmm(), 1, s, fmt)
    want = orc.split_fmm_dgemm(algs["222"], A, B, C.copy(order="F"), s, 0.5, -1.25, fmt=fmt)
    assert np.array_equal(got, want)
    assert fmm.take_device_error() == 0


@pytest.mark.parametrize("fmt,s,levels", [("bf16", 6, 2), ("fp8", 10, 1), ("bf16", 4, 0)])
def test_host_call_equals_device_call(fmm, torch_cuda, fmt, s, levels):
    """2100 x 1900 x 1500 (pair tiles at levels 0 and 1): the same bits as
    the device-pointer call on the same values."""
    m, n, k = 2100, 1900, 1500
    A, B, C = rand(m, k, 511), rand(k, n, 512), rand(m, n, 513)
    f = fmm.strassen_fmm() if levels else None
    want = device_call(fmm, f, levels, A, B, C, s, fmt)
    got = C.copy(order="F")
    fmm.split_strassen_ab_ex(1.0, A, B, 1.0, got, f, levels, s, fmt)
    assert np.array_equal(got, want)


def test_host_call_pinned_tensors_and_leading_dims(fmm, torch_cuda):
    """Pinned CPU tensors; operands that are column blocks of larger arrays
    (leading dimension > rows) through the C ABI."""
    import ctypes
    import torch
    m, n, k = 700, 500, 900
    A, B, C = rand(m, k, 521), rand(k, n, 522), rand(m, n, 523)
    want = device_call(fmm, fmm.strassen_fmm(), 1, A, B, C, 5, "bf16", 2.0, 0.5)
    hA = torch.from_numpy(A.T.copy()).pin_memory().t()
    hB = torch.from_numpy(B.T.copy()).pin_memory().t()
    hC = torch.from_numpy(C.T.copy()).pin_memory().t()
    fmm.split_strassen_ab_ex(2.0, hA, hB, 0.5, hC, fmm.strassen_fmm(), 1, 5, "bf16")
    assert np.array_equal(hC.numpy(), want)
    # leading dimensions larger than the row counts
    Ab = np.zeros((m + 9, k), order="F"); Ab[:m] = A
    Bb = np.zeros((k + 3, n), order="F"); Bb[:k] = B
    Cb = np.full((m + 5, n), 7.0, order="F"); Cb[:m] = C
    L = fmm.lib()
    st = L.fmm_gpu_split_strassen_ab_ex(2.0, Ab.ctypes.data, m + 9, Bb.ctypes.data, k + 3, 0.5, Cb.ctypes.data,
                                        m + 5, m, n, k, fmm.strassen_fmm(), 1, 5, 0)
    assert st == 0
    assert np.array_equal(Cb[:m], want)
    assert np.all(Cb[m:] == 7.0)


def test_host_call_scalar_cases(fmm, torch_cuda):
    m, n, k = 130, 70, 90
    A, B, C = rand(m, k, 531), rand(k, n, 532), rand(m, n, 533)
    f = fmm.strassen_fmm()
    # beta = 0: C's old values (NaN here) are not read
    Cn = np.full((m, n), np.nan, order="F")
    fmm.split_strassen_ab_ex(1.0, A, B, 0.0, Cn, f, 1, 6)
    assert np.array_equal(Cn, device_call(fmm, f, 1, A, B, np.zeros((m, n), order="F"), 6, "bf16", 1.0, 0.0))
    # alpha = 0 and k = 0: C := beta*C
    Cs = C.copy(order="F")
    fmm.split_strassen_ab_ex(0.0, A, B, -2.0, Cs, f, 1, 6)
    assert np.array_equal(Cs, -2.0 * C)
    Ck = C.copy(order="F")
    fmm.split_strassen_ab_ex(1.0, np.zeros((m, 0), order="F"), np.zeros((0, n), order="F"), 3.0, Ck, f, 1, 6)
    assert np.array_equal(Ck, 3.0 * C)
    # m = 0: nothing to do
    fmm.split_strassen_ab_ex(1.0, np.zeros((0, k), order="F"), B, 1.0, np.zeros((0, n), order="F"), f, 1, 6)
    fmm.release_host_buffers()
    assert fmm.take_device_error() == 0


@pytest.mark.parametrize("fmt,s", [("bf16", 6), ("fp8", 10)])
def test_host_call_any_layout(fmm, torch_cuda, fmt, s):
    """Row-major A, a transposed view for B, a strided view for C (general
    strides, like BLIS obj_t): the same bits as the Fortran-order call."""
    m, n, k = 300, 170, 260
    A, B, C = rand(m, k, 541), rand(k, n, 542), rand(m, n, 543)
    f = fmm.strassen_fmm()
    want = C.copy(order="F")
    fmm.split_strassen_ab_ex(0.5, A, B, 2.0, want, f, 1, s, fmt)
    Ar = np.ascontiguousarray(A)                       # row-major
    Bt = np.asfortranarray(B.T).T                      # transposed view (row-major storage of B)
    big = np.full((2 * m, 3 * n), 9.0)
    Cv = big[::2, ::3]                                 # general strides
    Cv[...] = C
    fmm.split_strassen_ab_ex(0.5, Ar, Bt, 2.0, Cv, f, 1, s, fmt)
    assert np.array_equal(Cv, want)
    mask = np.ones_like(big, dtype=bool)
    mask[::2, ::3] = False
    assert np.all(big[mask] == 9.0)                    # only C's own elements written


def test_host_call_timeline(fmm):
    """The host-buffer call's timeline (CUDA events inside the call): A and
    B are on the device before the GEMM ends (the blocked schedule starts the
    GEMM on half of each), the GEMM ends before C's last chunk is back, and
    the device span fits inside the call's host wall time."""
    import torch
    assert torch.cuda.is_available()
    m, n, k = 1500, 1300, 1100
    A, B, C = rand(m, k, 71), rand(k, n, 72), rand(m, n, 73)
    f = fmm.strassen_fmm()
    fmm.set_host_timeline(True)
    try:
        fmm.split_strassen_ab_ex(1.0, A, B, 1.0, C.copy(order="F"), f, 1, 6)
    finally:
        fmm.set_host_timeline(False)
    t = fmm.read_host_timeline()
    assert set(t) == {"a_up", "b_up", "gemm_start", "gemm_end", "c_down", "host_wall"}
    assert 0.0 < t["a_up"] <= t["gemm_end"] and 0.0 < t["b_up"] <= t["gemm_end"]
    assert 0.0 < t["gemm_start"] < t["gemm_end"] <= t["c_down"] <= t["host_wall"]


def test_host_alloc_buffers(fmm, torch_cuda):
    """Operands in the library's pinned huge-page host memory (fmm.host_empty,
    fmm_gpu_host_alloc): zeroed, page-locked for the GPU, usable as numpy
    arrays and torch CPU tensors by the host-buffer calls with the device
    call's bits, and freed once the last view is gone."""
    import gc

    import torch
    m, n, k = 700, 650, 900
    A, B, C = rand(m, k, 81), rand(k, n, 82), rand(m, n, 83)
    hA, hB, hC = fmm.host_empty(m, k), fmm.host_empty(k, n), fmm.host_empty(m, n)
    assert hA.flags.f_contiguous and not hA.any()
    hA[:], hB[:], hC[:] = A, B, C
    assert torch.from_numpy(hA).is_pinned()
    f = fmm.strassen_fmm()
    fmm.split_strassen_ab_ex(1.0, hA, hB, 1.0, hC, f, 1, 6)
    assert np.array_equal(hC, device_call(fmm, f, 1, A, B, C, 6, "bf16"))
    tC = torch.from_numpy(fmm.host_empty(m, n))
    tC.numpy()[:] = C
    fmm.split_strassen_ab_ex(1.0, torch.from_numpy(hA), torch.from_numpy(hB), 1.0, tC, f, 1, 6)
    assert np.array_equal(tC.numpy(), hC)
    # a buffer larger than a huge page
    big = fmm.host_empty(8192, 8192)
    assert big.shape == (8192, 8192) and torch.from_numpy(big).is_pinned()
    del hA, hB, hC, tC, big
    gc.collect()
    assert fmm.take_device_error() == 0


@pytest.mark.parametrize("levels,shape,alpha,beta", [(1, (517, 1033, 700), 1.5, 0.5), (2, (1037, 1033, 411), 1.0, 0.0),
                                                     (0, (300, 2311, 257), -1.0, 2.0), (1, (200, 1033, 300), 1.0, 1.0),
                                                     (1, (1033, 200, 300), 0.5, 1.0)])
def test_host_call_gemm_blocks(fmm, torch_cuda, levels, shape, alpha, beta):
    """Product grids of at least two GEMM tiles along a side run the GEMM in
    up to 2 x 2 blocks (A row halves, B column halves), each block's C
    elements updated and read back during the next block (uneven halves such
    as 259 / 3 rows and 517 / 3 columns of the product grid; row halves only;
    column halves only; leading dimensions larger than the row counts): the
    device call's bits."""
    m, n, k = shape
    A, B, C = rand(m, k, 551), rand(k, n, 552), rand(m, n, 553)
    f = fmm.strassen_fmm() if levels else None
    want = device_call(fmm, f, levels, A, B, C, 6, "bf16", alpha, beta)
    Ab = np.zeros((m + 3, k), order="F"); Ab[:m] = A
    Cb = np.full((m + 7, n), 5.0, order="F"); Cb[:m] = C
    L = fmm.lib()
    st = L.fmm_gpu_split_strassen_ab_ex(alpha, Ab.ctypes.data, m + 3, B.ctypes.data, k, beta, Cb.ctypes.data, m + 7,
                                        m, n, k, f if f is not None else fmm.FmmT(), levels, 6, 0)
    assert st == 0
    assert np.array_equal(Cb[:m], want)
    assert np.all(Cb[m:] == 5.0)
    got = C.copy(order="F")
    fmm.split_strassen_ab_ex(alpha, A, B, beta, got, f, levels, 6)
    assert np.array_equal(got, want)
    assert fmm.take_device_error() == 0
