"""Split-precision form on the GPU: bit-exact against the oracle's
restatement of the same integer/FP64 arithmetic (digits, exact chunk sums,
64-bit level accumulation, FP64 recombination), plus accuracy properties."""
import numpy as np
import pytest

from conftest import ALGS, COEFFS, rand
from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def run_split(fmm, f, levels, A, B, C, s, alpha=1.0, beta=1.0):
    dC = to_dev(C)
    fmm.split_dgemm(to_dev(A), to_dev(B), dC, f, levels, s, alpha=alpha, beta=beta)
    return to_host(dC)


@pytest.mark.parametrize("alg", ALGS)
@pytest.mark.parametrize("shape", [(1, 1, 1), (3, 13, 7), (65, 70, 33), (200, 130, 301)])
@pytest.mark.parametrize("s", [3, 6])
def test_split_bitexact_one_level(fmm, orc, algs, torch_cuda, alg, shape, s):
    m, n, k = shape
    A, B, C = rand(m, k, 51), rand(k, n, 52), rand(m, n, 53)
    f = fmm.new_fmm(COEFFS / f"{alg}.txt")
    try:
        got = run_split(fmm, f, 1, A, B, C, s)
    finally:
        fmm.free_fmm(f)
    want = orc.split_fmm_dgemm(algs[alg], A, B, C.copy(order="F"), s)
    assert np.array_equal(got, want), float(np.max(np.abs(got - want)))


@pytest.mark.parametrize("s", [2, 4, 5, 7, 8])
def test_split_bitexact_all_slice_counts(fmm, orc, algs, torch_cuda, s):
    A, B, C = rand(150, 260, 61), rand(260, 140, 62), rand(150, 140, 63)
    f = fmm.strassen_fmm()
    got = run_split(fmm, f, 1, A, B, C, s)
    want = orc.split_fmm_dgemm(algs["222"], A, B, C.copy(order="F"), s)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("alg", ["222", "333"])
def test_split_bitexact_two_levels(fmm, orc, algs, torch_cuda, alg):
    from oracle import coeffs as oc
    A, B, C = rand(300, 280, 71), rand(280, 310, 72), rand(300, 310, 73)
    f = fmm.new_fmm(COEFFS / f"{alg}.txt")
    try:
        got = run_split(fmm, f, 2, A, B, C, 6)
    finally:
        fmm.free_fmm(f)
    want = orc.split_fmm_dgemm(oc.power(algs[alg], 2), A, B, C.copy(order="F"), 6)
    assert np.array_equal(got, want)


def test_split_classical_and_scalars(fmm, orc, torch_cuda):
    from oracle import coeffs as oc
    A, B, C = rand(129, 257, 81), rand(257, 131, 82), rand(129, 131, 83)
    for alpha, beta in [(1.0, 1.0), (2.0, 0.0), (-0.75, 0.5)]:
        got = run_split(fmm, None, 0, A, B, C, 7, alpha, beta)
        want = orc.split_fmm_dgemm(oc.classical(), A, B, C.copy(order="F"), 7, alpha, beta)
        assert np.array_equal(got, want)


def test_split_long_k_chunks(fmm, orc, algs, torch_cuda):
    """k spanning many 256-term chunks and more than one TMEM buffer pass."""
    A, B, C = rand(128, 4100, 91), rand(4100, 128, 92), rand(128, 128, 93)
    f = fmm.strassen_fmm()
    got = run_split(fmm, f, 1, A, B, C, 6)
    want = orc.split_fmm_dgemm(algs["222"], A, B, C.copy(order="F"), 6)
    assert np.array_equal(got, want)


def test_split_worst_case_chunk_sums(fmm, orc, algs, torch_cuda):
    """All-equal operands: every digit product has the same sign, so each
    1024-term chunk reaches 2^24, the largest magnitude the exact FP32 path
    allows."""
    A = np.asfortranarray(np.full((128, 2048), -0.99999999999))
    B = np.asfortranarray(np.full((2048, 128), 0.99999999999))
    C = np.zeros((128, 128), order="F")
    for s in (2, 6, 8):
        got = run_split(fmm, None, 0, A, B, C, s)
        want = orc.split_fmm_dgemm((1, 1, 1, 1, np.ones((1, 1)), np.ones((1, 1)), np.ones((1, 1))), A, B,
                                   C.copy(order="F"), s)
        assert np.array_equal(got, want)


def test_split_hard_case_accuracy(fmm, torch_cuda):
    from fmm_blis_gb300 import synth
    A, B = synth.hard(192, 200, 5, 4.0), synth.hard(200, 180, 6, 4.0)
    C = np.zeros((192, 180), order="F")
    f = fmm.strassen_fmm()
    ref = A @ B
    dC = to_dev(C)
    fmm.dgemm(to_dev(A), to_dev(B), dC, f, 1)
    err64 = float(np.max(np.abs(to_host(dC) - ref)))
    got = run_split(fmm, f, 1, A, B, C, 7)
    assert float(np.max(np.abs(got - ref))) <= 10 * err64


def test_split_workspace_errors(fmm, torch_cuda):
    import ctypes
    import torch
    L = fmm.lib()
    A, B, C = to_dev(rand(64, 64, 1)), to_dev(rand(64, 64, 2)), to_dev(rand(64, 64, 3))
    need = fmm.split_workspace_size(64, 64, 64, None, 0, 6)
    ws = torch.empty(need, dtype=torch.uint8, device="cuda")
    assert L.fmm_gpu_split_dgemm(None, 0, 64, 64, 64, 1.0, A.data_ptr(), 64, B.data_ptr(), 64, 1.0, C.data_ptr(),
                                 64, 6, ws.data_ptr(), need - 256, None) == 9
    assert L.fmm_gpu_split_dgemm(None, 0, 64, 64, 64, 1.0, A.data_ptr(), 64, B.data_ptr(), 64, 1.0, C.data_ptr(),
                                 64, 9, ws.data_ptr(), need, None) == 1
    big_k = 16384 * 2 + 64
    assert fmm.split_workspace_size(8, 8, big_k, None, 0, 6) > 0
    assert L.fmm_gpu_take_device_error() == 0


def test_split_large_accuracy_vs_fp64(fmm, torch_cuda):
    """4096^3, two-level Strassen: 6- and 7-slice results against the plain
    FP64 FMM and the classical FP64 GEMM of this library."""
    import torch
    n = 4096
    g = torch.Generator(device="cuda").manual_seed(9)
    A = (torch.rand((n, n), generator=g, device="cuda", dtype=torch.float64) * 2 - 1).t()
    B = (torch.rand((n, n), generator=g, device="cuda", dtype=torch.float64) * 2 - 1).t()
    Cc = torch.zeros((n, n), device="cuda", dtype=torch.float64).t()
    fmm.dgemm(A, B, Cc, None, 0)
    f = fmm.strassen_fmm()
    Cf = torch.zeros_like(Cc)
    fmm.dgemm(A, B, Cf, f, 2)
    err_fmm = float((Cf - Cc).abs().max())
    Cs = torch.zeros_like(Cc)
    fmm.split_dgemm(A, B, Cs, f, 2, 7)
    err_split = float((Cs - Cc).abs().max())
    assert err_split <= 10 * err_fmm
