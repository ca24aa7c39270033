"""The CTA-pair GEMM (clusters of two CTAs, 256 x 256 tiles, tcgen05.mma
cta_group::2) that split calls use once m_e >= 1024: bit-exact against the
oracle and against the single-SM kernel, in single and batched calls."""
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


@pytest.mark.parametrize("fmt,s", [("bf16", 6), ("fp8", 9)])
def test_pair_classical_bitexact(fmm, orc, torch_cuda, fmt, s):
    from oracle import coeffs as oc
    m, n, k = 1100, 700, 300                  # m_e = 1100: pair tiles
    A, B, C = rand(m, k, 401), rand(k, n, 402), rand(m, n, 403)
    dC = to_dev(C)
    fmm.split_dgemm(to_dev(A), to_dev(B), dC, None, 0, s, fmt=fmt, alpha=0.75, beta=-0.5)
    want = orc.split_fmm_dgemm(oc.classical(), A, B, C.copy(order="F"), s, 0.75, -0.5, fmt=fmt)
    assert np.array_equal(to_host(dC), want)
    assert fmm.take_device_error() == 0


def test_pair_strassen_bitexact(fmm, orc, algs, torch_cuda):
    m, n, k = 2100, 600, 400                  # m_e = 1050: pair tiles, uneven parts
    A, B, C = rand(m, k, 411), rand(k, n, 412), rand(m, n, 413)
    dC = to_dev(C)
    fmm.split_dgemm(to_dev(A), to_dev(B), dC, fmm.strassen_fmm(), 1, 6)
    want = orc.split_fmm_dgemm(algs["222"], A, B, C.copy(order="F"), 6)
    assert np.array_equal(to_host(dC), want)


@pytest.mark.parametrize("fmt,s", [("bf16", 6), ("fp8", 10)])
def test_pair_equals_single_cta_kernel(fmm, torch_cuda, fmt, s):
    """4096^3, one Strassen level (m_e = 2048): the pair kernel and the
    single-SM kernel (pair tiles switched off) give the same bits."""
    import torch
    n = 4096
    g = torch.Generator(device="cuda").manual_seed(23)
    A = (torch.rand((n, n), generator=g, device="cuda", dtype=torch.float64) * 2 - 1).t()
    B = (torch.rand((n, n), generator=g, device="cuda", dtype=torch.float64) * 2 - 1).t()
    C1 = torch.zeros((n, n), device="cuda", dtype=torch.float64).t()
    C2 = torch.zeros_like(C1)
    f = fmm.strassen_fmm()
    fmm.split_dgemm(A, B, C1, f, 1, s, fmt=fmt)
    prev = fmm.set_split_pair_rows(2**31 - 1)
    try:
        fmm.split_dgemm(A, B, C2, f, 1, s, fmt=fmt)
    finally:
        fmm.set_split_pair_rows(prev)
    torch.cuda.synchronize()
    assert torch.equal(C1, C2)
    assert fmm.take_device_error() == 0


def test_batch_mixes_pair_and_single_launches(fmm, torch_cuda):
    """A batch with problems on both sides of the pair threshold (one wave,
    two GEMM launches) gives every problem its single-call bits."""
    import torch
    f = fmm.strassen_fmm()
    g = torch.Generator(device="cuda").manual_seed(31)
    shapes = [(2304, 1100, 700, "bf16", 5), (300, 200, 150, "fp8", 9), (2050, 2050, 260, "fp8", 10),
              (700, 500, 900, "bf16", 6), (1030, 300, 129, "bf16", 4)]
    probs, refs = [], []
    for i, (m, n, k, fmt, s) in enumerate(shapes):
        A = (torch.rand((k, m), generator=g, device="cuda", dtype=torch.float64) * 2 - 1).t()
        B = (torch.rand((n, k), generator=g, device="cuda", dtype=torch.float64) * 2 - 1).t()
        C0 = (torch.rand((n, m), generator=g, device="cuda", dtype=torch.float64) * 2 - 1).t()
        lv = 0 if i == 4 else 1
        probs.append({"A": A, "B": B, "C": C0.clone(), "fmm": f if lv else None, "levels": lv, "slices": s,
                      "fmt": fmt})
        Cr = C0.clone()
        fmm.split_dgemm(A, B, Cr, f if lv else None, lv, s, fmt=fmt)
        refs.append(Cr)
    fmm.batch_dgemm(probs)
    torch.cuda.synchronize()
    for i, (p, r) in enumerate(zip(probs, refs)):
        assert torch.equal(p["C"], r), f"problem {i}"
    assert fmm.take_device_error() == 0


def test_overlapped_groups_equal_one_group(fmm, torch_cuda):
    """8192 x 8192 x 512, two Strassen levels: with the recommended workspace
    the call runs its 49 products as two overlapping groups (group 2 packed
    beside group 1's GEMM, group 1's C updates beside group 2's GEMM); with a
    workspace just too small for that it runs them as one group. Same bits."""
    import torch
    n, k = 8192, 512
    g = torch.Generator(device="cuda").manual_seed(29)
    A = (torch.rand((k, n), generator=g, device="cuda", dtype=torch.float64) * 2 - 1).t()
    B = (torch.rand((n, k), generator=g, device="cuda", dtype=torch.float64) * 2 - 1).t()
    C0 = (torch.rand((n, n), generator=g, device="cuda", dtype=torch.float64) * 2 - 1).t()
    f = fmm.strassen_fmm()
    need = fmm.split_workspace_size(n, n, k, f, 2, 6)
    C1, C2 = C0.clone(), C0.clone()
    ws = torch.empty(need, dtype=torch.uint8, device="cuda")
    fmm.split_dgemm(A, B, C1, f, 2, 6, workspace=ws, alpha=0.5, beta=2.0)
    ws_one = torch.empty(need - (16 << 20), dtype=torch.uint8, device="cuda")
    fmm.split_dgemm(A, B, C2, f, 2, 6, workspace=ws_one, alpha=0.5, beta=2.0)
    torch.cuda.synchronize()
    assert torch.equal(C1, C2)
    assert fmm.take_device_error() == 0


def test_short_launches_equal_one_launch(fmm, torch_cuda):
    """16384 x 16384 x 128, two Strassen levels (m_e = 4096, 256 pair tiles per
    product): the single call runs each product group's GEMM as several
    back-to-back launches; a one-problem batch covers all 49 products in one
    launch. Same bits."""
    import torch
    n, k = 16384, 128
    g = torch.Generator(device="cuda").manual_seed(31)
    A = (torch.rand((k, n), generator=g, device="cuda", dtype=torch.float64) * 2 - 1).t()
    B = (torch.rand((n, k), generator=g, device="cuda", dtype=torch.float64) * 2 - 1).t()
    C0 = (torch.rand((n, n), generator=g, device="cuda", dtype=torch.float64) * 2 - 1).t()
    f = fmm.strassen_fmm()
    C1, C2 = C0.clone(), C0.clone()
    fmm.read_kernel_timing()
    fmm.set_kernel_timing(True)
    try:
        fmm.split_dgemm(A, B, C1, f, 2, 6, alpha=-1.5, beta=0.5)
        torch.cuda.synchronize()
        _, launches, products = fmm.read_kernel_timing()
    finally:
        fmm.set_kernel_timing(False)
    assert products == 49 and launches > 2
    fmm.batch_dgemm([{"A": A, "B": B, "C": C2, "fmm": f, "levels": 2, "slices": 6, "alpha": -1.5, "beta": 0.5}])
    torch.cuda.synchronize()
    assert torch.equal(C1, C2)
    assert fmm.take_device_error() == 0
