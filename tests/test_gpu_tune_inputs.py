"""Input-aware slice choice (Tuner.plan_for) on config 3's input classes:
uniform [-1, 1) and (u - 0.5) exp(phi g) with phi = 1 and 4. The plan it
picks for a relative max-norm target of 1e-10 must meet that target against
the classical FP64 GEMM; uniform inputs keep the shape plan's slice count,
wide-range inputs get more slices where the shape plan would miss."""
import pytest

from conftest import COEFFS
from gpu_util import to_dev

pytestmark = pytest.mark.gpu

TARGET = 1e-10


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def operands(kind, n):
    from fmm_blis_gb300 import synth
    if kind == "uniform":
        return synth.uniform(n, n, 41), synth.uniform(n, n, 42)
    phi = {"phi1": 1.0, "phi4": 4.0}[kind]
    return synth.hard(n, n, 41, phi), synth.hard(n, n, 42, phi)


def run_plan(fmm, p, A, B, torch):
    f = None if p.alg == "classical" else fmm.new_fmm(COEFFS / f"{p.alg}.txt")
    try:
        C = torch.zeros((B.shape[1], A.shape[0]), dtype=torch.float64, device="cuda").t()
        fmm.split_dgemm(A, B, C, f, p.levels, p.slices, fmt=p.fmt)
        torch.cuda.synchronize()
        return C
    finally:
        if f is not None:
            fmm.free_fmm(f)


@pytest.mark.parametrize("kind", ["uniform", "phi1", "phi4"])
def test_plan_for_meets_the_target(fmm, torch_cuda, kind):
    from fmm_blis_gb300 import tune
    torch = torch_cuda
    n = 2048
    hA, hB = operands(kind, n)
    A, B = to_dev(hA), to_dev(hB)
    tuner = tune.Tuner()
    shape = tuner.plan(n, n, n, "split", TARGET)
    p = tuner.plan_for(fmm, A, B, TARGET)
    assert (p.alg, p.levels, p.fmt) == (shape.alg, shape.levels, shape.fmt)
    ref = torch.zeros((n, n), dtype=torch.float64, device="cuda").t()
    fmm.dgemm(A, B, ref, None, 0)
    rel = float((run_plan(fmm, p, A, B, torch) - ref).abs().max()) / float(ref.abs().max())
    assert rel <= TARGET, (kind, p, rel)
    if kind == "uniform":
        assert p.slices == shape.slices
    if kind == "phi4":
        # the shape plan alone would miss the target on these inputs
        rel_shape = float((run_plan(fmm, shape, A, B, torch) - ref).abs().max()) / float(ref.abs().max())
        assert p.slices > shape.slices and rel_shape > TARGET, (shape, rel_shape)
    assert fmm.take_device_error() == 0
