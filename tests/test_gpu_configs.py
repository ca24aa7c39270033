"""Parity at the benchmark configurations' sizes, against the oracle.

- Strassen 222 at one level, m=n=k=2048, FP64: GPU against the oracle's FMM
  on the whole matrix (conftest.C_BOUND).
- Every coefficient file at two levels, m=n=k=4096, FP64: the same.
- Rectangular (m, k, n) = (16384, 4096, 16384), 444 at two levels, FP64: a
  slab of C rows against the oracle's classical FP64 product of those rows
  (the FMM's whole error, also within C_BOUND's c).
- Split BF16, Strassen at two levels, m=n=k=16384, 6 slices (the headline
  workload): bit for bit against the oracle's restatement on sampled rows of
  the product grid (each lands on one C row per part row, all columns).
"""
import numpy as np
import pytest

from conftest import C_BOUND, COEFFS, fmm_bound, rand
from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def alg_power(name, levels):
    from oracle import coeffs as oc
    return oc.power(oc.read(COEFFS / f"{name}.txt"), levels)


def fmm_levels(fmm, name):
    return fmm.new_fmm(COEFFS / f"{name}.txt")


@pytest.mark.parametrize("alg,levels,n", [("222", 1, 2048), ("222", 2, 4096), ("232", 2, 4096),
                                          ("322", 2, 4096), ("333", 2, 4096), ("444", 2, 4096)])
def test_fp64_config_size_matches_oracle(fmm, orc, torch_cuda, alg, levels, n):
    A, B, C = rand(n, n, 901), rand(n, n, 902), rand(n, n, 903)
    f = fmm_levels(fmm, alg)
    try:
        dC = to_dev(C)
        fmm.dgemm(to_dev(A), to_dev(B), dC, f, levels)
        got = to_host(dC)
    finally:
        fmm.free_fmm(f)
    want = orc.fmm_dgemm(alg_power(alg, levels), A, B, C.copy(order="F"))
    assert np.max(np.abs(got - want)) <= fmm_bound(A, B, C, n, C_BOUND[(alg, levels)])


def test_fp64_rectangular_row_slab_matches_classical_oracle(fmm, orc, torch_cuda):
    m, k, n = 16384, 4096, 16384
    A, B = rand(m, k, 911), rand(k, n, 912)
    f = fmm_levels(fmm, "444")
    try:
        dC = to_dev(np.zeros((m, n), order="F"))
        fmm.dgemm(to_dev(A), to_dev(B), dC, f, 2)
        rows = np.r_[0:32, 8190:8194, m - 32:m]
        got = dC[rows].cpu().numpy()
    finally:
        fmm.free_fmm(f)
    want = orc.dgemm(np.asfortranarray(A[rows]), B, np.zeros((len(rows), n), order="F"))
    assert np.max(np.abs(got - want)) <= fmm_bound(A, B, np.zeros(1), k, C_BOUND[("444", 2)])


def test_split_headline_bit_exact_on_sampled_rows(fmm, orc, torch_cuda):
    import torch
    n, s = 16384, 6
    A, B, C = rand(n, n, 921), rand(n, n, 922), rand(n, n, 923)
    a = alg_power("222", 2)
    f = fmm.strassen_fmm()
    dC = to_dev(C)
    fmm.split_dgemm(to_dev(A), to_dev(B), dC, f, 2, s)
    torch.cuda.synchronize()
    me = n // a[0]
    local = [0, 1, me // 2 + 7, me - 1]
    rows = sorted({r for i in local for r in orc.part_rows(n, a[0], i)})
    got = dC[rows].cpu().numpy()
    del dC
    want = orc.split_fmm_dgemm_rows(a, A, B, C.copy(order="F"), s, local)
    assert len(rows) == 4 * len(local)
    assert np.array_equal(got, want[rows])
