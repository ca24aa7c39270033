"""Tuner (per-problem plan choice) and the served request generator: host
logic only, no GPU."""
import pytest

from fmm_blis_gb300 import serve, tune


@pytest.fixture(scope="module")
def tuner():
    return tune.Tuner()


def test_alg_shapes_from_coefficient_files():
    shapes = {(a.name, a.levels): a for a in tune.alg_shapes()}
    s222 = shapes[("222", 1)]
    assert (s222.mt, s222.kt, s222.nt, s222.R, s222.nnz_w) == (2, 2, 2, 7, 12)
    assert shapes[("222", 2)].R == 49 and shapes[("222", 2)].nnz_w == 144
    assert (shapes[("232", 1)].mt, shapes[("232", 1)].kt, shapes[("232", 1)].nt) == (2, 3, 2)
    assert shapes[("444", 2)].R == 2401


def test_model_matches_calibration_points():
    """The cost model reproduces the GB300 measurements it was fitted to
    (m = n = k = 16384) within 10%."""
    a = {(x.name, x.levels): x for x in tune.alg_shapes()}
    n = 16384
    assert tune.fp64_time(a[("classical", 0)], n, n, n) == pytest.approx(7.03, rel=0.1)
    assert tune.fp64_time(a[("444", 2)], n, n, n) == pytest.approx(5.24, rel=0.1)
    assert tune.fp64_time(a[("333", 2)], n, n, n) == pytest.approx(5.86, rel=0.1)
    assert tune.fp64_time(a[("444", 1)], n, n, n) == pytest.approx(5.62, rel=0.1)
    assert tune.split_time(a[("222", 2)], n, n, n, 6) == pytest.approx(0.105, rel=0.1)


def test_plans(tuner):
    p = tuner.plan(16384, 16384, 16384, "fp64")
    assert (p.form, p.levels, p.slices) == ("fp64", 2, 0) and p.alg in ("444", "222", "333")
    p = tuner.plan(16384, 16384, 16384, "split", 1e-10)
    assert p.form == "split" and p.levels >= 1 and 5 <= p.slices <= 7
    # small or skinny shapes stay classical
    for shp in [(256, 256, 256), (128, 16384, 128), (300, 200, 100)]:
        assert tuner.plan(*shp, "fp64").levels == 0
        assert tuner.plan(*shp, "split", 1e-10).levels == 0
    # deterministic and cached
    assert tuner.plan(5000, 3000, 7000, "split", 1e-10) is tuner.plan(5000, 3000, 7000, "split", 1e-10)


def test_slices_follow_target(tuner):
    prev = None
    for tol in (1e-6, 1e-8, 1e-10, 1e-12, 1e-14):
        p = tuner.plan(4096, 4096, 4096, "split", tol)
        assert p.est_rel_err * tune.ERR_SAFETY <= tol
        if prev is not None:
            assert p.slices >= prev
        prev = p.slices
    with pytest.raises(ValueError):
        tuner.plan(4096, 4096, 4096, "split", 1e-30)


def test_poisson_arrivals_seeded():
    a = serve.poisson_arrivals(1000.0, 2.0, seed=3, cap_bytes=8 * 3 * 4096 ** 2)
    b = serve.poisson_arrivals(1000.0, 2.0, seed=3, cap_bytes=8 * 3 * 4096 ** 2)
    assert [(r.m, r.n, r.k, r.form, r.seed, r.arrival) for r in a] == \
           [(r.m, r.n, r.k, r.form, r.seed, r.arrival) for r in b]
    assert 1700 < len(a) < 2300                      # rate x duration
    assert all(8 * (r.m * r.k + r.k * r.n + r.m * r.n) <= 8 * 3 * 4096 ** 2 for r in a)
    assert all(0 < r.arrival <= 2.0 for r in a)
    assert {r.form for r in a} == {"split", "fp64"}


def test_batch_sizing_needs_no_gpu():
    """Workspace sizing of a batch problem reads shapes only (host tables)."""
    import fmm_blis_gb300 as fmm
    f = fmm.strassen_fmm()
    sizes = [fmm.batch_problem_workspace_size(1000, 900, 800, f, 1, s) for s in (3, 5, 7)]
    assert 0 < sizes[0] < sizes[1] < sizes[2]
    assert fmm.batch_problem_workspace_size(100, 90, 80, None, 0, 5) > 0
    # a whole batch from its shapes and plans (what the server sizes its arena pieces with): at least
    # each problem's own workspace, and the FP64 problems' table beside the split problems'
    shapes = [(1000, 900, 800, f, 1, 5, "bf16"), (300, 200, 700, None, 0, 6, "bf16"), (512, 512, 512, f, 1, 0, "bf16")]
    whole = fmm.batch_shapes_workspace_size(shapes)
    assert whole >= max(fmm.batch_problem_workspace_size(*p) for p in shapes)
    assert whole == fmm.batch_shapes_workspace_size(list(shapes))
    assert fmm.batch_shapes_workspace_size([]) >= 0


def test_slice_format_choice():
    """Both slice formats are candidates; the FP8 error model uses 5 bits per
    slice and its pair cost the measured 0.55 of a BF16 pair."""
    t = tune.Tuner()
    p = t.plan(16384, 16384, 16384, "split", 1e-10)
    fmts = {c.fmt for c in p.candidates}
    assert fmts == {"bf16", "fp8"}
    fp8 = [c for c in p.candidates if c.fmt == "fp8"]
    assert all(c.slices >= 8 for c in fp8)
    only8 = tune.Tuner(formats=("fp8",)).plan(16384, 16384, 16384, "split", 1e-10)
    assert only8.fmt == "fp8" and only8.est_rel_err * tune.ERR_SAFETY <= 1e-10
    a = {(x.name, x.levels): x for x in tune.alg_shapes()}
    assert tune.split_time(a[("222", 2)], 16384, 16384, 16384, 10, "fp8") == pytest.approx(0.157, rel=0.15)


def test_small_skinny_classical_model():
    """Classical FP64 problems with a small output and a long k are modelled
    on the small/skinny cluster path (k split over CTAs): measured on GB300
    128 x 128 x 16384 in 1.05 ms and 256 x 256 x 8192 in 1.06 ms (against 4.44
    and 2.23 ms with one CTA per 32 x 32 tile down all of k)."""
    a = {(x.name, x.levels): x for x in tune.alg_shapes()}
    cls = a[("classical", 0)]
    assert tune.fp64_time(cls, 128, 128, 16384) == pytest.approx(1.05e-3, rel=0.2)
    assert tune.fp64_time(cls, 256, 256, 8192) == pytest.approx(1.06e-3, rel=0.2)
    # the same output with a short k stays on the regular kernel
    assert tune._sup_splits(128, 128, 300) == 0
    p = tune.Tuner().plan(128, 128, 16384, "fp64")
    assert (p.alg, p.levels) == ("classical", 0)
