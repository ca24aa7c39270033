"""Batched execution (fmm_gpu_batch_dgemm): every problem of a batch of
uneven GEMMs -- mixed algorithms, levels, slice counts and plain FP64
problems -- must give bit for bit what its own single call gives."""
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


def single(fmm, p):
    dC = to_dev(p["C0"])
    if p["slices"]:
        fmm.split_dgemm(p["A"], p["B"], dC, p["fmm"], p["levels"], p["slices"], alpha=p["alpha"], beta=p["beta"])
    else:
        fmm.dgemm(p["A"], p["B"], dC, p["fmm"], p["levels"], alpha=p["alpha"], beta=p["beta"])
    return to_host(dC)


def make_problems(fmm, seed, count):
    rng = np.random.default_rng(seed)
    algs = {a: fmm.new_fmm(COEFFS / f"{a}.txt") for a in ("222", "232", "333")}
    probs = []
    for i in range(count):
        m, n, k = (int(x) for x in np.exp(rng.uniform(np.log(8), np.log(700), 3)))
        choice = rng.integers(0, 5)
        f, levels = [(None, 0), (algs["222"], 1), (algs["222"], 2), (algs["232"], 1), (algs["333"], 1)][choice]
        slices = int(rng.choice([0, 3, 5, 6, 7])) if i % 4 else 0
        C0 = rand(m, n, 1000 + i)
        probs.append({"A": to_dev(rand(m, k, 2000 + i)), "B": to_dev(rand(k, n, 3000 + i)), "C0": C0,
                      "C": to_dev(C0), "fmm": f, "levels": levels, "slices": slices,
                      "alpha": float(rng.choice([1.0, -0.5])), "beta": float(rng.choice([1.0, 0.0, 2.0]))})
    return probs, algs


@pytest.mark.parametrize("ws_scale", [1.0, 0.3, 0.02])   # one wave; waves over two halves; many waves
def test_batch_bitexact_vs_single_calls(fmm, torch_cuda, ws_scale):
    import torch
    probs, algs = make_problems(fmm, 7, 40)
    try:
        batch = fmm.make_batch(probs)
        need = fmm.batch_workspace_size(batch)
        ws = torch.empty(max(int(need * ws_scale), 1 << 20), dtype=torch.uint8, device="cuda")
        if ws_scale < 1.0:
            # small workspace: many waves, the largest problems run alone
            ws = torch.empty(max(int(need * ws_scale), 64 << 20), dtype=torch.uint8, device="cuda")
        fmm.batch_dgemm(batch, workspace=ws)
        torch.cuda.synchronize()
        for i, p in enumerate(probs):
            want = single(fmm, p)
            assert np.array_equal(to_host(p["C"]), want), f"problem {i}"
        assert fmm.take_device_error() == 0
    finally:
        for f in algs.values():
            fmm.free_fmm(f)


def test_batch_empty_and_degenerate(fmm, torch_cuda):
    import torch
    fmm.batch_dgemm([])
    C0 = rand(5, 4, 1)
    p = {"A": to_dev(np.zeros((5, 0), order="F")), "B": to_dev(np.zeros((0, 4), order="F")), "C": to_dev(C0),
         "fmm": fmm.strassen_fmm(), "levels": 1, "slices": 6, "beta": 3.0}
    fmm.batch_dgemm([p])
    torch.cuda.synchronize()
    assert np.array_equal(to_host(p["C"]), 3.0 * C0)


def test_batch_all_fp64_one_launch(fmm, torch_cuda):
    """Plain FP64 problems of a batch run in one persistent launch (a work
    queue over (problem, tile position) items; small/skinny classical
    problems in their own cluster launches) and match their single calls bit
    for bit, including the degenerate ones (k = 0, alpha = 0, beta = 0)."""
    import torch
    rng = np.random.default_rng(11)
    algs = {a: fmm.new_fmm(COEFFS / f"{a}.txt") for a in ("222", "322", "444")}
    cases = [(None, 0), (algs["222"], 1), (algs["222"], 2), (algs["322"], 1), (algs["444"], 1), (algs["444"], 2)]
    probs = []
    try:
        for i in range(48):
            m, n, k = (int(x) for x in np.exp(rng.uniform(np.log(4), np.log(600), 3)))
            if i == 5:
                k = 0
            f, levels = cases[i % len(cases)]
            C0 = rand(m, n, 500 + i)
            probs.append({"A": to_dev(rand(m, k, 600 + i)), "B": to_dev(rand(k, n, 700 + i)), "C0": C0,
                          "C": to_dev(C0), "fmm": f, "levels": levels, "slices": 0,
                          "alpha": 0.0 if i == 7 else float(rng.choice([1.0, 0.75])),
                          "beta": float(rng.choice([1.0, 0.0, -1.5]))})
        n0 = fmm.launch_count()
        fmm.batch_dgemm(probs)
        torch.cuda.synchronize()
        launches = fmm.launch_count() - n0
        # table writer + the batch kernel, plus the small/skinny classical
        # problems' own launches (C := beta*C when beta != 1, then the cluster kernel)
        sup = [p for p in probs if p["fmm"] is None and p["alpha"] != 0.0 and
               fmm.f64_sup_splits(p["A"].shape[0], p["B"].shape[1], p["A"].shape[1])]
        assert launches <= 2 + sum(1 + (p["beta"] != 1.0) for p in sup), launches
        for i, p in enumerate(probs):
            assert np.array_equal(to_host(p["C"]), single(fmm, p)), f"problem {i}"
        assert fmm.take_device_error() == 0
    finally:
        for f in algs.values():
            fmm.free_fmm(f)


def test_batch_more_problems_than_one_launch(fmm, torch_cuda):
    """More split problems than one GEMM launch's table holds: consecutive
    waves, each result still equal to its single call."""
    import torch
    f = fmm.strassen_fmm()
    probs = []
    for i in range(100):
        m, n, k = 40 + (i * 7) % 90, 30 + (i * 11) % 100, 50 + (i * 13) % 120
        C0 = rand(m, n, 900 + i)
        probs.append({"A": to_dev(rand(m, k, 1900 + i)), "B": to_dev(rand(k, n, 2900 + i)), "C0": C0,
                      "C": to_dev(C0), "fmm": f, "levels": 1 if i % 3 else 0, "slices": 3 + i % 5,
                      "alpha": 1.0, "beta": 1.0})
    for p in probs:
        if p["levels"] == 0:
            p["fmm"] = None
    fmm.batch_dgemm(probs)
    torch.cuda.synchronize()
    for i, p in enumerate(probs):
        assert np.array_equal(to_host(p["C"]), single(fmm, p)), f"problem {i}"
    assert fmm.take_device_error() == 0


def test_batch_wave_side_work_in_few_launches(fmm, torch_cuda):
    """A wave's side work runs as one launch per kernel over all its problems
    (per slice kind for the packs): BF16 and FP8 slices of several counts,
    one and two levels, and a 444 two-level problem whose 256 C sub-blocks
    take the per-problem C-update form. Every result equals its single call."""
    import torch
    algs = {a: fmm.new_fmm(COEFFS / f"{a}.txt") for a in ("222", "444")}
    rng = np.random.default_rng(21)
    kinds = [("bf16", 5), ("bf16", 6), ("fp8", 10)]
    probs = []
    try:
        for i in range(30):
            m, n, k = (int(x) for x in rng.integers(60, 500, 3))
            fmt, s = kinds[i % 3]
            f, levels = [(None, 0), (algs["222"], 1), (algs["222"], 2)][i % 3 if i % 5 else 1]
            if i == 29:
                f, levels, fmt, s, (m, n, k) = algs["444"], 2, "bf16", 6, (200, 180, 170)
            C0 = rand(m, n, 4000 + i)
            probs.append({"A": to_dev(rand(m, k, 5000 + i)), "B": to_dev(rand(k, n, 6000 + i)), "C0": C0,
                          "C": to_dev(C0), "fmm": f, "levels": levels, "slices": s, "fmt": fmt,
                          "alpha": float(rng.choice([1.0, 0.5])), "beta": float(rng.choice([1.0, 0.0, -2.0]))})
        n0 = fmm.launch_count()
        fmm.batch_dgemm(probs)
        torch.cuda.synchronize()
        launches = fmm.launch_count() - n0
        assert launches <= 16, launches       # one wave: 3 + 2 x 3 kinds + GEMMs + C updates
        for i, p in enumerate(probs):
            dC = to_dev(p["C0"])
            fmm.split_dgemm(p["A"], p["B"], dC, p["fmm"], p["levels"], p["slices"], alpha=p["alpha"], beta=p["beta"],
                            fmt=p["fmt"])
            assert np.array_equal(to_host(p["C"]), to_host(dC)), f"problem {i}"
        assert fmm.take_device_error() == 0
    finally:
        for f in algs.values():
            fmm.free_fmm(f)
