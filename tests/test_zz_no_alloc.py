"""The allocation-free split entry point (fmm_gpu_split_dgemm_noalloc).

It exists for callers that cannot allocate device memory while they run: a
plug-in working in memory that its host application's allocator owns, a
process whose device memory is already reserved, a loop that cannot afford
cudaFree's implicit device synchronization. Instead of a caller workspace it
uses the library's static 64 MiB device scratch. These tests call it through
the C ABI and require the same bits as the workspace entry point, on two calls
in a row (the scratch keeps the previous call's contents, so the second call
checks that nothing stale leaks into its result), and require the device's
free memory to be the same before and after calls."""
import ctypes

import numpy as np
import pytest

from conftest import COEFFS, rand
from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu

FMM_ERR_SCRATCH = 10


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def call_noalloc(fmm, f, levels, A, B, C, s, alpha=1.0, beta=1.0):
    L = fmm.lib()
    m, k = A.shape
    n = B.shape[1]
    pf = ctypes.byref(f) if f is not None else None
    return L.fmm_gpu_split_dgemm_noalloc(pf, levels, m, n, k, alpha, A.data_ptr(), m, B.data_ptr(), k, beta,
                                         C.data_ptr(), m, s, None)


@pytest.mark.parametrize("alg,levels,shape,s", [("222", 1, (300, 260, 410), 6), ("333", 1, (129, 200, 97), 7),
                                                ("222", 2, (260, 300, 280), 5), (None, 0, (200, 150, 333), 8)])
def test_noalloc_matches_workspace_entry_twice(fmm, torch_cuda, alg, levels, shape, s):
    import torch
    f = fmm.new_fmm(COEFFS / f"{alg}.txt") if alg else None
    try:
        m, n, k = shape
        for call in range(2):
            A, B, C = rand(m, k, 100 + call), rand(k, n, 200 + call), rand(m, n, 300 + call)
            dA, dB = to_dev(A), to_dev(B)
            ref = to_dev(C)
            fmm.split_dgemm(dA, dB, ref, f, levels, s, alpha=1.25, beta=0.5)
            got = to_dev(C)
            assert call_noalloc(fmm, f, levels, dA, dB, got, s, 1.25, 0.5) == 0
            torch.cuda.synchronize()
            assert np.array_equal(to_host(got), to_host(ref)), f"call {call}"
    finally:
        if f is not None:
            fmm.free_fmm(f)


def test_noalloc_rejects_problems_beyond_the_scratch(fmm, torch_cuda):
    import torch
    n = 8192
    A = torch.zeros((n, n), dtype=torch.float64, device="cuda").t()
    C = torch.zeros((n, n), dtype=torch.float64, device="cuda").t()
    assert call_noalloc(fmm, None, 0, A, A, C, 6) == FMM_ERR_SCRATCH
    assert fmm.take_device_error() == 0


def test_noalloc_leaves_device_memory_unchanged(fmm, torch_cuda):
    import torch
    m, n, k = 700, 650, 900
    A, B, C = rand(m, k, 11), rand(k, n, 12), rand(m, n, 13)
    dA, dB = to_dev(A), to_dev(B)
    ref, got = to_dev(C), to_dev(C)
    fmm.split_dgemm(dA, dB, ref, None, 0, 6)
    fmm.split_dgemm(dA, dB, ref, None, 0, 6)
    warm = to_dev(C)
    assert call_noalloc(fmm, None, 0, dA, dB, warm, 6) == 0   # loads the kernels before the count starts
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        assert call_noalloc(fmm, None, 0, dA, dB, got, 6) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert np.array_equal(to_host(got), to_host(ref))
    assert fmm.take_device_error() == 0
