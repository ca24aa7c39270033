"""Plain FP64 form on the FP64 tensor-core path (fmm_gpu_set_f64_engine
FMM_F64_MMA: mma.sync m8n8k4 f64 over the same fused-pack tiles as the DFMA
micro-kernel). Same bound against the oracle (conftest.C_BOUND) and against
the reference's own outputs; batched problems give their single calls' bits
on this engine too."""
import numpy as np
import pytest

from conftest import ALGS, C_BOUND, COEFFS, fmm_bound, rand
from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1, 1), (3, 13, 7), (17, 9, 23), (64, 64, 64), (130, 67, 95), (257, 129, 300), (700, 650, 900)]


@pytest.fixture
def mma_engine(fmm):
    import torch
    assert torch.cuda.is_available()
    prev = fmm.set_f64_engine("mma")
    yield
    fmm.set_f64_engine(prev)


@pytest.mark.parametrize("alg", ALGS)
@pytest.mark.parametrize("levels", [1, 2])
@pytest.mark.parametrize("shape", SHAPES)
def test_mma_engine_matches_oracle(fmm, orc, algs, mma_engine, alg, levels, shape):
    from oracle import coeffs as oc
    m, n, k = shape
    A, B, C = rand(m, k, 51), rand(k, n, 52), rand(m, n, 53)
    f = fmm.new_fmm(COEFFS / f"{alg}.txt")
    try:
        dC = to_dev(C)
        fmm.dgemm(to_dev(A), to_dev(B), dC, f, levels, alpha=0.75, beta=1.25)
        got = to_host(dC)
    finally:
        fmm.free_fmm(f)
    want = orc.fmm_dgemm(oc.power(algs[alg], levels), A, B, C.copy(order="F"), alpha=0.75, beta=1.25)
    assert np.max(np.abs(got - want)) <= fmm_bound(0.75 * A, B, 1.25 * C, k, C_BOUND[(alg, levels)])


@pytest.mark.parametrize("shape", [(512, 512, 512), (1000, 300, 2000), (64, 3000, 64)])
def test_mma_engine_classical(fmm, orc, mma_engine, shape):
    m, n, k = shape
    A, B, C = rand(m, k, 61), rand(k, n, 62), rand(m, n, 63)
    dC = to_dev(C)
    fmm.dgemm(to_dev(A), to_dev(B), dC, None, 0)
    want = orc.dgemm(A, B, C.copy(order="F"))
    assert np.max(np.abs(to_host(dC) - want)) <= fmm_bound(A, B, C, k, 2)


def test_mma_engine_batch_equals_single_calls(fmm, mma_engine):
    import torch
    rng = np.random.default_rng(17)
    algs = {a: fmm.new_fmm(COEFFS / f"{a}.txt") for a in ("222", "333")}
    cases = [(None, 0), (algs["222"], 1), (algs["222"], 2), (algs["333"], 1)]
    probs = []
    try:
        for i in range(20):
            m, n, k = (int(x) for x in np.exp(rng.uniform(np.log(8), np.log(500), 3)))
            f, levels = cases[i % len(cases)]
            C0 = rand(m, n, 800 + i)
            probs.append({"A": to_dev(rand(m, k, 900 + i)), "B": to_dev(rand(k, n, 1000 + i)), "C0": C0,
                          "C": to_dev(C0), "fmm": f, "levels": levels, "slices": 0,
                          "alpha": float(rng.choice([1.0, -0.5])), "beta": float(rng.choice([1.0, 0.0, 2.0]))})
        fmm.batch_dgemm(probs)
        torch.cuda.synchronize()
        for i, p in enumerate(probs):
            dC = to_dev(p["C0"])
            fmm.dgemm(p["A"], p["B"], dC, p["fmm"], p["levels"], alpha=p["alpha"], beta=p["beta"])
            assert np.array_equal(to_host(p["C"]), to_host(dC)), f"problem {i}"
    finally:
        for f in algs.values():
            fmm.free_fmm(f)


def test_mma_engine_matches_reference_outputs(fmm, mma_engine):
    from ref_fixtures import FULL, case
    for name in FULL:
        meta, A, B, C, z = case(name)
        f = fmm.new_fmm(COEFFS / f"{meta['alg']}.txt")
        try:
            dC = to_dev(C)
            fmm.dgemm(to_dev(A), to_dev(B), dC, f, meta["levels"])
            got = to_host(dC)
        finally:
            fmm.free_fmm(f)
        bound = fmm_bound(A, B, C, meta["k"], C_BOUND[(meta["alg"], meta["levels"])])
        assert np.max(np.abs(got - z["C_ref"])) <= bound, name
