"""Served form: continuous batching with HBM admission, overlapping batches on
a stream pool and per-bucket CUDA graphs. Each request's result must be the
same bits whether it is served alone or in a mix, and equal to the single
call with its plan."""
import numpy as np
import pytest

from fmm_blis_gb300 import serve, tune

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def mix(seed, count):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(count):
        if i % 5 == 0:
            m, n, k = (int(x) for x in rng.integers(2500, 3200, 3))     # FMM plans
        else:
            m, n, k = (int(x) for x in np.exp(rng.uniform(np.log(16), np.log(1000), 3)))
        reqs.append(serve.Request(m, n, k, form="split" if i % 3 else "fp64", target_rel_err=1e-10,
                                  seed=1000 + i, arrival=0.001 * i))
    return reqs


def small_tuner():
    # FMM levels from 512-sized sub-blocks so the mix holds FMM plans at modest sizes
    return tune.Tuner(min_block_fp64=512, min_block_split=512)


def host(t):
    return t.cpu().numpy()


def direct(fmm, torch, r, algs):
    """the request computed by the single call of its plan"""
    g = torch.Generator(device="cuda").manual_seed(r.seed)
    A = serve._colmajor_rand(torch, r.m, r.k, g, torch.device("cuda"))
    B = serve._colmajor_rand(torch, r.k, r.n, g, torch.device("cuda"))
    C = serve._colmajor_rand(torch, r.m, r.n, g, torch.device("cuda"))
    p = r.plan
    f = None if p.alg == "classical" else algs.setdefault(p.alg, fmm.new_fmm(tune.COEFF_DIR / f"{p.alg}.txt"))
    if p.form == "fp64":
        fmm.dgemm(A, B, C, f, p.levels)
    else:
        fmm.split_dgemm(A, B, C, f, p.levels, p.slices, fmt=p.fmt)
    torch.cuda.synchronize()
    return host(C)


def test_served_mix_equals_alone_and_direct(fmm, torch_cuda):
    torch = torch_cuda
    tuner = small_tuner()
    reqs = mix(5, 30)
    srv = serve.Server(streams=3, tuner=tuner, max_batch=6)
    done = srv.run(reqs)
    srv.close()
    assert len(done) == len(reqs)
    assert srv.launched_batches >= 2
    paths = {r.path for r in reqs}
    assert paths == {"batch", "graph"}, paths
    assert any(r.plan.levels > 0 for r in reqs)
    mixed = {r.seed: host(r.C) for r in reqs}
    algs = {}
    try:
        for r in mix(5, 30):
            alone = serve.Server(streams=1, tuner=tuner)
            alone.run([serve.Request(r.m, r.n, r.k, r.form, r.target_rel_err, r.seed, 0.0)])
            (a,) = alone.completed
            alone.close()
            assert np.array_equal(host(a.C), mixed[r.seed]), (r.m, r.n, r.k, r.form, a.path)
            assert np.array_equal(direct(fmm, torch, a, algs), mixed[r.seed]), (r.m, r.n, r.k, r.form, a.path)
    finally:
        for f in algs.values():
            fmm.free_fmm(f)
    assert fmm.take_device_error() == 0


def test_admission_respects_hbm_budget(fmm, torch_cuda):
    reqs = [serve.Request(900, 800, 700 + 10 * i, form="split", seed=i, arrival=0.0) for i in range(12)]
    probe = serve.Server(streams=2, use_graphs=False)
    one = probe.submit(serve.Request(900, 800, 820, form="split", seed=99)).footprint
    probe.pending.clear()
    probe.close()
    srv = serve.Server(hbm_budget=int(2.5 * one), streams=2, use_graphs=False)
    srv.run(reqs)
    srv.close()
    assert len(srv.completed) == 12
    assert srv.peak_used <= srv.budget
    assert srv.launched_batches >= 6          # at most two requests fit at a time
    with pytest.raises(ValueError):
        srv.submit(serve.Request(4096, 4096, 4096, form="split"))


def test_split_plans_meet_their_target(fmm, torch_cuda):
    """The tuner's slice choice keeps the max-norm error relative to max|C|
    under the requested target (uniform inputs, FP64 classical reference)."""
    torch = torch_cuda
    tuner = small_tuner()
    algs = {}
    try:
        for (m, n, k), tol in [((1500, 1300, 2100), 1e-10), ((700, 900, 1100), 1e-8), ((2048, 2048, 2048), 1e-12)]:
            r = serve.Request(m, n, k, "split", tol, seed=m)
            r.plan = tuner.plan(m, n, k, "split", tol)
            got = direct(fmm, torch, r, algs)
            g = torch.Generator(device="cuda").manual_seed(r.seed)
            A = serve._colmajor_rand(torch, m, k, g, torch.device("cuda"))
            B = serve._colmajor_rand(torch, k, n, g, torch.device("cuda"))
            C = serve._colmajor_rand(torch, m, n, g, torch.device("cuda"))
            fmm.dgemm(A, B, C, None, 0)
            ref = host(C)
            rel = np.abs(got - ref).max() / np.abs(ref).max()
            assert rel <= tol, (m, n, k, tol, r.plan, rel)
    finally:
        for f in algs.values():
            fmm.free_fmm(f)
