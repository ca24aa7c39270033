"""Small/skinny classical path of the plain FP64 form (the BLIS "sup"
counterpart, blis/kernels/haswell/3/sup): a classical FP64 GEMM with a small
output and a long k runs as clusters of CTAs that split k into chunks and add
the chunk partials through distributed shared memory in chunk order.

Its result is checked against the oracle's classical GEMM within the same
bound as the regular kernel (the two differ only in the order of the k sum),
and the batched call must give the single call's bits for such problems."""
import numpy as np
import pytest

from conftest import fmm_bound, rand
from gpu_util import to_dev, to_host

SUP_SHAPES = [(128, 128, 16384), (100, 90, 5000), (33, 700, 3000), (64, 64, 600), (257, 129, 2048), (1, 1, 1024)]


def test_sup_split_rule(fmm):
    """The chunk count is a function of the shape only (no GPU needed)."""
    assert fmm.f64_sup_splits(128, 128, 16384) == 8
    assert fmm.f64_sup_splits(33, 700, 3000) == 5        # 2 x 22 tiles: 256 CTAs at most
    assert fmm.f64_sup_splits(100, 90, 5000) == 8        # 4 x 3 tiles, 96 CTAs
    assert fmm.f64_sup_splits(64, 64, 600) == 2          # k / 256 limits the chunks
    assert fmm.f64_sup_splits(257, 129, 2048) == 5       # 9 x 5 tiles: 256 / 45
    assert fmm.f64_sup_splits(288, 512, 8192) == 0       # 9 x 16 tiles: more than 128
    assert fmm.f64_sup_splits(128, 128, 300) == 0        # too short a k
    assert fmm.f64_sup_splits(512, 512, 4096) == 0       # 256 tiles: the regular kernel fills the GPU
    assert fmm.f64_sup_splits(0, 10, 4096) == 0


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


@pytest.mark.gpu
@pytest.mark.parametrize("shape", SUP_SHAPES)
@pytest.mark.parametrize("alpha,beta", [(1.0, 1.0), (-0.75, 0.5), (2.0, 0.0)])
def test_sup_matches_oracle(fmm, orc, torch_cuda, shape, alpha, beta):
    m, n, k = shape
    A, B, C = rand(m, k, 51), rand(k, n, 52), rand(m, n, 53)
    dC = to_dev(C)
    n0 = fmm.launch_count()
    fmm.dgemm(to_dev(A), to_dev(B), dC, None, 0, alpha=alpha, beta=beta)
    launches = fmm.launch_count() - n0
    want = orc.dgemm(A, B, C.copy(order="F"), alpha, beta)
    got = to_host(dC)
    assert np.max(np.abs(got - want)) <= fmm_bound(alpha * A, B, beta * C, k, 2)
    ks = fmm.f64_sup_splits(m, n, k)
    if ks:   # one cluster launch (plus C := beta*C when beta != 1)
        assert launches == 1 + (beta != 1.0), launches
    assert fmm.take_device_error() == 0


@pytest.mark.gpu
def test_sup_batch_equals_single_calls(fmm, torch_cuda):
    """Small/skinny classical problems inside a batch take the same kernel as
    their single calls: same bits, next to regular FP64 and split problems."""
    import torch
    f = fmm.strassen_fmm()
    shapes = SUP_SHAPES + [(300, 280, 400), (90, 80, 700)]
    probs = []
    for i, (m, n, k) in enumerate(shapes):
        C0 = rand(m, n, 800 + i)
        probs.append({"A": to_dev(rand(m, k, 810 + i)), "B": to_dev(rand(k, n, 820 + i)), "C0": C0,
                      "C": to_dev(C0), "fmm": None, "levels": 0, "slices": 0,
                      "alpha": 1.5 if i % 2 else 1.0, "beta": 0.25 if i % 3 == 1 else 1.0})
    probs.append({"A": to_dev(rand(200, 300, 1)), "B": to_dev(rand(300, 150, 2)), "C0": rand(200, 150, 3),
                  "C": None, "fmm": f, "levels": 1, "slices": 6, "alpha": 1.0, "beta": 1.0})
    probs[-1]["C"] = to_dev(probs[-1]["C0"])
    fmm.batch_dgemm(probs)
    torch.cuda.synchronize()
    for i, p in enumerate(probs):
        dC = to_dev(p["C0"])
        if p["slices"]:
            fmm.split_dgemm(p["A"], p["B"], dC, p["fmm"], p["levels"], p["slices"], alpha=p["alpha"], beta=p["beta"])
        else:
            fmm.dgemm(p["A"], p["B"], dC, p["fmm"], p["levels"], alpha=p["alpha"], beta=p["beta"])
        assert np.array_equal(to_host(p["C"]), to_host(dC)), f"problem {i}"
    assert fmm.take_device_error() == 0


@pytest.mark.gpu
def test_sup_same_bits_with_either_engine(fmm, torch_cuda):
    """The small/skinny path has one micro-kernel (DFMA), whichever engine the
    regular kernel is set to."""
    m, n, k = 128, 128, 16384
    A, B, C = to_dev(rand(m, k, 61)), to_dev(rand(k, n, 62)), rand(m, n, 63)
    out = []
    for engine in ("dfma", "mma"):
        prev = fmm.set_f64_engine(engine)
        try:
            dC = to_dev(C)
            fmm.dgemm(A, B, dC, None, 0)
            out.append(to_host(dC))
        finally:
            fmm.set_f64_engine(prev)
    assert np.array_equal(out[0], out[1])
