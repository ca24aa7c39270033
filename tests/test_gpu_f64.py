"""Plain FP64 form on the GPU against the oracle (same algorithm, same inputs).

Bound: max|C_gpu - C_oracle| <= c * eps64 * k * max|A| * max|B| (+ 4 eps max|C0|),
with c per (algorithm, levels) from conftest.C_BOUND. The two sides differ only in
the order of the k-sums of each product, so c stays small."""
import numpy as np
import pytest

from conftest import ALGS, C_BOUND, COEFFS, GOLDEN, fmm_bound, rand
from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1, 1), (3, 13, 7), (17, 9, 23), (64, 64, 64), (130, 67, 95), (257, 129, 300)]


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


@pytest.mark.parametrize("alg", ALGS)
@pytest.mark.parametrize("levels", [1, 2])
@pytest.mark.parametrize("shape", SHAPES)
def test_fmm_f64_matches_oracle(fmm, orc, algs, torch_cuda, alg, levels, shape):
    from oracle import coeffs as oc
    m, n, k = shape
    A, B, C = rand(m, k, 31), rand(k, n, 32), rand(m, n, 33)
    f = fmm.new_fmm(COEFFS / f"{alg}.txt")
    try:
        dC = to_dev(C)
        fmm.dgemm(to_dev(A), to_dev(B), dC, f, levels)
        got = to_host(dC)
    finally:
        fmm.free_fmm(f)
    want = orc.fmm_dgemm(oc.power(algs[alg], levels), A, B, C.copy(order="F"))
    assert np.max(np.abs(got - want)) <= fmm_bound(A, B, C, k, C_BOUND[(alg, levels)])


@pytest.mark.parametrize("shape", SHAPES + [(512, 512, 512)])
def test_classical_f64_matches_oracle(fmm, orc, torch_cuda, shape):
    m, n, k = shape
    A, B, C = rand(m, k, 41), rand(k, n, 42), rand(m, n, 43)
    dC = to_dev(C)
    fmm.dgemm(to_dev(A), to_dev(B), dC, None, 0)
    want = orc.dgemm(A, B, C.copy(order="F"))
    assert np.max(np.abs(to_host(dC) - want)) <= fmm_bound(A, B, C, k, 2)


def test_reference_kat_through_host_dropin(fmm, orc, algs, torch_cuda):
    """test/test_strassen_oapi.c:44-242 through the host-buffer drop-in
    (bli_strassen_ab_ex replacement): Frobenius residual against my_mm."""
    g = np.load(GOLDEN / "kat_3x13x7.npz")
    A, B, C = (np.asfortranarray(g[x]) for x in "ABC")
    f = fmm.new_fmm(COEFFS / "222.txt")
    try:
        Cg = C.copy(order="F")
        fmm.bli_strassen_ab_ex(1.0, A, B, 1.0, Cg, f)
    finally:
        fmm.free_fmm(f)
    C_ref = orc.naive_dgemm(A, B, C.copy(order="F"))
    assert np.linalg.norm(Cg - C_ref) <= 1e-7
    assert np.max(np.abs(Cg - g["C_out"])) <= 8 * np.finfo(float).eps * np.max(np.abs(g["C_out"]))


def test_strassen_ab_builtin(fmm, torch_cuda):
    A, B, C = rand(50, 40, 1), rand(40, 60, 2), rand(50, 60, 3)
    Cg = C.copy(order="F")
    st = fmm.lib().fmm_gpu_strassen_ab(1.0, A.ctypes.data, 50, B.ctypes.data, 40, 1.0, Cg.ctypes.data, 50,
                                       50, 60, 40)
    assert st == 0
    assert np.max(np.abs(Cg - (C + A @ B))) <= 1e-13


@pytest.mark.parametrize("alpha,beta", [(2.0, 0.0), (-0.5, 3.0), (1.0, 0.0), (0.0, 2.0), (1.5, 1.0)])
def test_alpha_beta(fmm, orc, algs, torch_cuda, alpha, beta):
    A, B, C = rand(70, 50, 4), rand(50, 66, 5), rand(70, 66, 6)
    f = fmm.new_fmm(COEFFS / "333.txt")
    try:
        dC = to_dev(C)
        fmm.dgemm(to_dev(A), to_dev(B), dC, f, 1, alpha=alpha, beta=beta)
    finally:
        fmm.free_fmm(f)
    want = beta * C + alpha * (A @ B)
    assert np.max(np.abs(to_host(dC) - want)) <= 1e-13


def test_strided_views(fmm, torch_cuda):
    """Leading dimensions larger than the row count (sub-matrix views)."""
    import torch
    A, B, C = rand(90, 70, 7), rand(70, 80, 8), rand(90, 80, 9)
    big = torch.zeros((128, 200), dtype=torch.float64, device="cuda").t().contiguous().t()
    dA = big[:90, :70]
    dA.copy_(to_dev(A))
    dC = torch.zeros((100, 80), dtype=torch.float64, device="cuda").t().contiguous().t()[:90]
    dC.copy_(to_dev(C))
    f = fmm.strassen_fmm()
    fmm.dgemm(dA, to_dev(B), dC, f, 1)
    assert np.max(np.abs(to_host(dC) - (C + A @ B))) <= 1e-13


def test_empty_and_errors(fmm, torch_cuda):
    import ctypes
    L = fmm.lib()
    f = fmm.strassen_fmm()
    # empty dimensions are no-ops
    assert L.fmm_gpu_dgemm(ctypes.byref(f), 1, 0, 5, 5, 1.0, None, 1, None, 5, 1.0, None, 1, None) == 0
    # k == 0 only scales C by beta
    C = rand(6, 5, 1)
    dC = to_dev(C)
    assert L.fmm_gpu_dgemm(ctypes.byref(f), 1, 6, 5, 0, 1.0, None, 6, None, 1, 2.0, dC.data_ptr(), 6, None) == 0
    assert np.array_equal(to_host(dC), 2.0 * C)
    # bad leading dimension
    assert L.fmm_gpu_dgemm(ctypes.byref(f), 1, 6, 5, 4, 1.0, dC.data_ptr(), 3, dC.data_ptr(), 4, 1.0,
                           dC.data_ptr(), 6, None) == 1


@pytest.mark.parametrize("alg,levels", [("222", 1), ("222", 2), ("333", 1)])
def test_large_property_f64(fmm, torch_cuda, alg, levels):
    """2048^3: FMM against this library's classical FP64 GEMM on the GPU."""
    import torch
    n = 2048
    g = torch.Generator(device="cuda").manual_seed(5)
    A = (torch.rand((n, n), generator=g, device="cuda", dtype=torch.float64) * 2 - 1).t()
    B = (torch.rand((n, n), generator=g, device="cuda", dtype=torch.float64) * 2 - 1).t()
    C0 = torch.zeros((n, n), device="cuda", dtype=torch.float64).t()
    Cc = C0.clone()
    fmm.dgemm(A, B, Cc, None, 0)
    f = fmm.new_fmm(COEFFS / f"{alg}.txt")
    try:
        Cf = C0.clone()
        fmm.dgemm(A, B, Cf, f, levels)
    finally:
        fmm.free_fmm(f)
    err = float((Cf - Cc).abs().max())
    eps = float(np.finfo(np.float64).eps)
    assert err <= 4 * eps * n * levels * (2 if alg == "333" else 1)


@pytest.mark.parametrize("layout", ["c_order", "transposed_views", "strided_slices", "mixed"])
def test_host_dropin_any_layout(fmm, orc, torch_cuda, layout):
    """The host drop-in takes operands in any layout a BLIS obj_t can have
    (column-major, row-major, transposed, general strides): the result equals
    the column-major call's bit for bit, and only C's elements are written."""
    m, n, k = 70, 53, 91
    A, B, C = rand(m, k, 301), rand(k, n, 302), rand(m, n, 303)
    f = fmm.strassen_fmm()
    want = C.copy(order="F")
    fmm.bli_strassen_ab_ex(0.5, A.copy(order="F"), B.copy(order="F"), 1.5, want, f)
    if layout == "c_order":
        a, b = np.ascontiguousarray(A), np.ascontiguousarray(B)
        c_buf = np.ascontiguousarray(C)
        c = c_buf
    elif layout == "transposed_views":
        a, b = np.asfortranarray(A.T).T, np.asfortranarray(B.T).T     # row-major data seen through .T
        c_buf = np.asfortranarray(C.T)
        c = c_buf.T
    elif layout == "strided_slices":
        big_a = np.zeros((2 * m, 3 * k))
        big_a[::2, ::3] = A
        a = big_a[::2, ::3]
        big_b = np.zeros((3 * k, 2 * n), order="F")
        big_b[::3, ::2] = B
        b = big_b[::3, ::2]
        c_buf = np.full((2 * m, 2 * n), 7.0)
        c_buf[::2, ::2] = C
        c = c_buf[::2, ::2]
    else:
        a = np.ascontiguousarray(A)
        b = B.copy(order="F")
        c_buf = np.ascontiguousarray(C)
        c = c_buf
    fmm.bli_strassen_ab_ex(0.5, a, b, 1.5, c, f)
    assert np.array_equal(np.asarray(c), want)
    if layout == "strided_slices":
        mask = np.ones(c_buf.shape, bool)
        mask[::2, ::2] = False
        assert np.all(c_buf[mask] == 7.0)
