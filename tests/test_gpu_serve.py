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
    # in the mix, small split requests whose size bucket has no graph yet take the batched path while an FP64
    # batch runs; alone they take the graph path: both give the direct call's bits
    assert {r.path for r in reqs} <= {"batch", "graph"}
    assert any(r.plan.levels > 0 for r in reqs)
    mixed = {r.seed: host(r.C) for r in reqs}
    algs = {}
    alone_paths = set()
    try:
        for r in mix(5, 30):
            alone = serve.Server(streams=1, tuner=tuner)
            alone.run([serve.Request(r.m, r.n, r.k, r.form, r.target_rel_err, r.seed, 0.0)])
            (a,) = alone.completed
            alone.close()
            alone_paths.add(a.path)
            assert np.array_equal(host(a.C), mixed[r.seed]), (r.m, r.n, r.k, r.form, a.path)
            assert np.array_equal(direct(fmm, torch, a, algs), mixed[r.seed]), (r.m, r.n, r.k, r.form, a.path)
    finally:
        for f in algs.values():
            fmm.free_fmm(f)
    assert alone_paths == {"batch", "graph"}, alone_paths
    assert fmm.take_device_error() == 0


def test_admission_respects_hbm_budget(fmm, torch_cuda):
    reqs = [serve.Request(900, 800, 700 + 10 * i, form="split", seed=i, arrival=0.0) for i in range(12)]
    probe = serve.Server(streams=2, use_graphs=False)
    one = probe.submit(serve.Request(900, 800, 820, form="split", seed=99)).footprint
    for q in probe.queues.values():
        q.clear()
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


def test_workspace_allocation_failure_is_retried(fmm, torch_cuda):
    """A workspace allocation that fails (injected on the host) puts the
    batch back in its queue; the loop goes on and every request completes
    with the bits it gets without the fault."""
    torch = torch_cuda
    tuner = small_tuner()
    calls = {"n": 0}

    def fail_first_two(nbytes):
        calls["n"] += 1
        if calls["n"] <= 2:
            raise MemoryError(f"injected: workspace of {nbytes} bytes")

    reqs = [serve.Request(600 + 37 * i, 500 + 11 * i, 700 - 13 * i, form="split" if i % 4 else "fp64",
                          seed=500 + i, arrival=0.0) for i in range(8)]
    srv = serve.Server(streams=2, tuner=tuner, use_graphs=False, alloc_hook=fail_first_two)
    srv.run(reqs)
    srv.close()
    assert srv.alloc_failures == 2
    assert len(srv.completed) == len(reqs)
    algs = {}
    try:
        for r in reqs:
            assert np.array_equal(direct(fmm, torch, r, algs), host(r.C)), (r.m, r.n, r.k, r.form)
    finally:
        for f in algs.values():
            fmm.free_fmm(f)
    assert fmm.take_device_error() == 0


def test_cancelled_requests_leave_the_rest_unchanged(fmm, torch_cuda):
    torch = torch_cuda
    tuner = small_tuner()
    srv = serve.Server(streams=2, tuner=tuner)
    reqs = [srv.submit(serve.Request(300 + 50 * i, 280, 310, form="split", seed=700 + i)) for i in range(6)]
    assert srv.cancel(reqs[2].rid)                 # waiting: leaves its queue
    assert srv.tick() == 5
    assert srv.cancel(reqs[4].rid)                 # admitted: dropped when its batch completes
    assert not srv.cancel(10**6)
    srv.run([])
    srv.close()
    assert sorted(r.rid for r in srv.cancelled) == sorted([reqs[2].rid, reqs[4].rid])
    assert sorted(r.rid for r in srv.completed) == sorted(r.rid for i, r in enumerate(reqs) if i not in (2, 4))
    assert srv.used == 0 and srv.used_fp64 == 0
    algs = {}
    try:
        for r in srv.completed:
            assert np.array_equal(direct(fmm, torch, r, algs), host(r.C))
    finally:
        for f in algs.values():
            fmm.free_fmm(f)


def test_split_requests_pass_a_long_fp64_batch(fmm, torch_cuda):
    """Per-form queues and the FP64 batch's CTA cap: split requests that arrive
    behind a long FP64 request are admitted and finish while it still runs."""
    srv = serve.Server(streams=2, use_graphs=False)
    big = serve.Request(4096, 4096, 4096, form="fp64", seed=1, arrival=0.0)
    small = [serve.Request(700, 650, 720, form="split", seed=10 + i, arrival=0.001 * (i + 1)) for i in range(10)]
    srv.run([big] + small)
    srv.close()
    assert big.done is not None and all(r.done is not None for r in small)
    assert max(r.done for r in small) < big.done
    assert fmm.take_device_error() == 0
