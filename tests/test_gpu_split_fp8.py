"""FP8-E4M3 slices of the split form on the GPU: bit-exact against the
oracle's restatement (base-32 digits, exact chunk sums, 64-bit level
accumulation in units of level min(s+1, 10), FP64 recombination), plus mixed
BF16/FP8 batches and accuracy properties."""
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


def run_fp8(fmm, f, levels, A, B, C, s, alpha=1.0, beta=1.0):
    dC = to_dev(C)
    fmm.split_dgemm(to_dev(A), to_dev(B), dC, f, levels, s, alpha=alpha, beta=beta, fmt="fp8")
    return to_host(dC)


@pytest.mark.parametrize("alg", ALGS)
@pytest.mark.parametrize("shape", [(1, 1, 1), (3, 13, 7), (65, 70, 33), (200, 130, 301)])
@pytest.mark.parametrize("s", [4, 9])
def test_fp8_bitexact_one_level(fmm, orc, algs, torch_cuda, alg, shape, s):
    m, n, k = shape
    A, B, C = rand(m, k, 151), rand(k, n, 152), rand(m, n, 153)
    f = fmm.new_fmm(COEFFS / f"{alg}.txt")
    try:
        got = run_fp8(fmm, f, 1, A, B, C, s)
    finally:
        fmm.free_fmm(f)
    want = orc.split_fmm_dgemm(algs[alg], A, B, C.copy(order="F"), s, fmt="fp8")
    assert np.array_equal(got, want), float(np.max(np.abs(got - want)))


@pytest.mark.parametrize("s", [2, 3, 5, 6, 7, 8, 10, 11, 12])
def test_fp8_bitexact_all_slice_counts(fmm, orc, algs, torch_cuda, s):
    A, B, C = rand(150, 260, 161), rand(260, 140, 162), rand(150, 140, 163)
    got = run_fp8(fmm, fmm.strassen_fmm(), 1, A, B, C, s)
    want = orc.split_fmm_dgemm(algs["222"], A, B, C.copy(order="F"), s, fmt="fp8")
    assert np.array_equal(got, want)


@pytest.mark.parametrize("alg", ["222", "333"])
def test_fp8_bitexact_two_levels(fmm, orc, algs, torch_cuda, alg):
    from oracle import coeffs as oc
    A, B, C = rand(300, 280, 171), rand(280, 310, 172), rand(300, 310, 173)
    f = fmm.new_fmm(COEFFS / f"{alg}.txt")
    try:
        got = run_fp8(fmm, f, 2, A, B, C, 9)
    finally:
        fmm.free_fmm(f)
    want = orc.split_fmm_dgemm(oc.power(algs[alg], 2), A, B, C.copy(order="F"), 9, fmt="fp8")
    assert np.array_equal(got, want)


def test_fp8_classical_scalars_and_long_k(fmm, orc, torch_cuda):
    from oracle import coeffs as oc
    A, B, C = rand(129, 257, 181), rand(257, 131, 182), rand(129, 131, 183)
    for alpha, beta in [(1.0, 1.0), (2.0, 0.0), (-0.75, 0.5)]:
        got = run_fp8(fmm, None, 0, A, B, C, 8, alpha, beta)
        want = orc.split_fmm_dgemm(oc.classical(), A, B, C.copy(order="F"), 8, alpha, beta, fmt="fp8")
        assert np.array_equal(got, want)
    # k across many 2048-term chunks and a partial last stage row
    A, B, C = rand(128, 8300, 191), rand(8300, 128, 192), rand(128, 128, 193)
    got = run_fp8(fmm, fmm.strassen_fmm(), 1, A, B, C, 10)
    want = orc.split_fmm_dgemm(oc.read(COEFFS / "222.txt"), A, B, C.copy(order="F"), 10, fmt="fp8")
    assert np.array_equal(got, want)


def test_fp8_equal_operands(fmm, orc, torch_cuda):
    """All-equal operands: every digit product of a chunk has the same sign."""
    A = np.asfortranarray(np.full((128, 4096), -0.99999999999))
    B = np.asfortranarray(np.full((4096, 128), 0.99999999999))
    C = np.zeros((128, 128), order="F")
    one = (1, 1, 1, 1, np.ones((1, 1)), np.ones((1, 1)), np.ones((1, 1)))
    for s in (2, 7, 12):
        got = run_fp8(fmm, None, 0, A, B, C, s)
        want = orc.split_fmm_dgemm(one, A, B, C.copy(order="F"), s, fmt="fp8")
        assert np.array_equal(got, want)


def test_fp8_rejects_bad_slices(fmm, torch_cuda):
    L = fmm.lib()
    A, B, C = to_dev(rand(64, 64, 1)), to_dev(rand(64, 64, 2)), to_dev(rand(64, 64, 3))
    assert L.fmm_gpu_split_dgemm_fmt(None, 0, 64, 64, 64, 1.0, A.data_ptr(), 64, B.data_ptr(), 64, 1.0,
                                     C.data_ptr(), 64, 13, 1, None, 0, None) == 1
    assert L.fmm_gpu_split_dgemm_fmt(None, 0, 64, 64, 64, 1.0, A.data_ptr(), 64, B.data_ptr(), 64, 1.0,
                                     C.data_ptr(), 64, 6, 2, None, 0, None) == 1
    assert fmm.split_workspace_size(64, 64, 64, None, 0, 12, "fp8") > 0
    assert fmm.split_workspace_size(64, 64, 64, None, 0, 13, "fp8") == 0


def test_fp8_mixed_batch_bitexact(fmm, torch_cuda):
    """BF16 and FP8 problems in one batch (one persistent GEMM launch per
    wave, the MMA kind chosen per work item) give their single-call bits."""
    import torch
    f = fmm.strassen_fmm()
    probs = []
    for i in range(24):
        m, n, k = 50 + 13 * i, 40 + 17 * (i % 7), 60 + 29 * (i % 5)
        C0 = rand(m, n, 700 + i)
        fmt = "fp8" if i % 2 else "bf16"
        probs.append({"A": to_dev(rand(m, k, 800 + i)), "B": to_dev(rand(k, n, 900 + i)), "C0": C0, "C": to_dev(C0),
                      "fmm": f if i % 3 else None, "levels": 1 if i % 3 else 0,
                      "slices": (4 + i % 8) if fmt == "fp8" else (3 + i % 5), "fmt": fmt})
    fmm.batch_dgemm(probs)
    torch.cuda.synchronize()
    for i, p in enumerate(probs):
        dC = to_dev(p["C0"])
        fmm.split_dgemm(p["A"], p["B"], dC, p["fmm"], p["levels"], p["slices"], fmt=p["fmt"])
        torch.cuda.synchronize()
        assert np.array_equal(to_host(p["C"]), to_host(dC)), f"problem {i}"
    assert fmm.take_device_error() == 0


def test_fp8_accuracy_vs_fp64(fmm, torch_cuda):
    """2048^3, one Strassen level: FP8 slices reach the FP64 FMM's accuracy
    with 11 slices (55 bits of digits)."""
    import torch
    n = 2048
    g = torch.Generator(device="cuda").manual_seed(19)
    A = (torch.rand((n, n), generator=g, device="cuda", dtype=torch.float64) * 2 - 1).t()
    B = (torch.rand((n, n), generator=g, device="cuda", dtype=torch.float64) * 2 - 1).t()
    Cc = torch.zeros((n, n), device="cuda", dtype=torch.float64).t()
    fmm.dgemm(A, B, Cc, None, 0)
    f = fmm.strassen_fmm()
    Cf = torch.zeros_like(Cc)
    fmm.dgemm(A, B, Cf, f, 1)
    err_fmm = float((Cf - Cc).abs().max())
    errs = {}
    for s in (7, 9, 11):
        Cs = torch.zeros_like(Cc)
        fmm.split_dgemm(A, B, Cs, f, 1, s, fmt="fp8")
        errs[s] = float((Cs - Cc).abs().max())
    assert errs[7] > errs[9] > errs[11]
    assert errs[11] <= 10 * err_fmm, (errs, err_fmm)
    assert fmm.take_device_error() == 0
