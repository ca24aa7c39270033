"""Failure detection without a GPU fault.

Every wait in the library's kernels is bounded: after its limit the waiting
thread records an error code in the device error word, makes the CTA's other
waiters give up, and the kernel ends. The self-test entry runs that path on
purpose -- a wait on a barrier nothing arrives at -- and the test checks the
status the host reads, that every thread gave up, that the word is cleared,
and that the library keeps computing correct results afterwards."""
import time

import numpy as np
import pytest

from conftest import rand
from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu

FMM_ERR_DEVICE = 8


def test_bounded_wait_expires_and_reports(fmm, orc):
    import torch
    assert torch.cuda.is_available()
    t0 = time.perf_counter()
    status, gave_up = fmm.selftest_wait_expiry()
    elapsed = time.perf_counter() - t0
    assert status == FMM_ERR_DEVICE
    assert gave_up == 64
    assert 1.5 < elapsed < 30.0          # the 2 s limit, not a hang
    assert fmm.take_device_error() == 0  # the synchronous read already cleared it
    # the context is usable: a split call right after gives the oracle's bits
    from oracle import coeffs as oc
    from conftest import COEFFS
    m, n, k = 150, 140, 170
    A, B, C = rand(m, k, 1), rand(k, n, 2), rand(m, n, 3)
    f = fmm.strassen_fmm()
    dC = to_dev(C)
    fmm.split_dgemm(to_dev(A), to_dev(B), dC, f, 1, 6)
    want = orc.split_fmm_dgemm(oc.read(COEFFS / "222.txt"), A, B, C.copy(order="F"), 6)
    assert np.array_equal(to_host(dC), want)
    assert fmm.take_device_error() == 0
