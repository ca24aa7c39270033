"""The oracle (CPU restatement of the reference FMM path) pinned against the
reference's own known-answer test and exact golden vectors, and the split-form
restatement's accuracy."""
import numpy as np
import pytest

from conftest import ALGS, GOLDEN, fmm_bound, rand


def test_reference_kat_3x13x7(orc, algs):
    """test/test_strassen_oapi.c:44-242: m=3 n=13 k=7, 222.txt, FMM against the
    naive loop my_mm; the reference gates the Frobenius residual at 1e-7."""
    g = np.load(GOLDEN / "kat_3x13x7.npz")
    A, B, C = (np.asfortranarray(g[x]) for x in "ABC")
    C_fmm = orc.fmm_dgemm(algs["222"], A, B, C.copy(order="F"))
    C_ref = orc.naive_dgemm(A, B, C.copy(order="F"))
    resid = np.linalg.norm(C_fmm - C_ref)
    assert resid <= 1e-7
    assert resid <= 1e-14
    assert np.max(np.abs(C_fmm - g["C_out"])) <= 8 * np.finfo(float).eps * np.max(np.abs(g["C_out"]))


@pytest.mark.parametrize("name", ["exact_17x9x23", "exact_33x31x40"])
@pytest.mark.parametrize("alg", ALGS)
def test_oracle_against_exact_golden(orc, algs, name, alg):
    g = np.load(GOLDEN / f"{name}.npz")
    A, B, C = (np.asfortranarray(g[x]) for x in "ABC")
    out = orc.fmm_dgemm(algs[alg], A, B, C.copy(order="F"))
    k = A.shape[1]
    assert np.max(np.abs(out - g["C_out"])) <= fmm_bound(A, B, C, k, 16)


@pytest.mark.parametrize("alg", ALGS)
@pytest.mark.parametrize("levels", [1, 2])
@pytest.mark.parametrize("shape", [(1, 1, 1), (5, 3, 2), (37, 29, 41), (64, 64, 64), (70, 33, 96)])
def test_oracle_fmm_matches_classical(orc, algs, alg, levels, shape):
    from oracle import coeffs as oc
    if levels == 2 and alg == "444" and max(shape) < 64:
        pytest.skip("444 two-level splits each dimension 16 ways")
    m, n, k = shape
    A, B, C = rand(m, k, 11), rand(k, n, 12), rand(m, n, 13)
    flat = oc.power(algs[alg], levels)
    out = orc.fmm_dgemm(flat, A, B, C.copy(order="F"))
    ref = C + A @ B
    assert np.max(np.abs(out - ref)) <= fmm_bound(A, B, C, k, 32 * levels)


def test_oracle_alpha_beta(orc, algs):
    A, B, C = rand(20, 18, 1), rand(18, 22, 2), rand(20, 22, 3)
    for alpha, beta in [(2.0, 0.0), (-0.5, 3.0), (1.0, 0.0), (0.0, 2.0)]:
        out = orc.fmm_dgemm(algs["222"], A, B, C.copy(order="F"), alpha, beta)
        ref = beta * C + alpha * (A @ B)
        assert np.max(np.abs(out - ref)) <= 1e-13


def test_oracle_products_subset_sums_to_whole(orc, algs):
    A, B, C = rand(40, 36, 4), rand(36, 44, 5), rand(40, 44, 6)
    whole = orc.fmm_dgemm(algs["333"], A, B, C.copy(order="F"))
    part = C.copy(order="F")
    orc.fmm_dgemm(algs["333"], A, B, part, r_begin=0, r_end=10)
    orc.fmm_dgemm(algs["333"], A, B, part, r_begin=10, r_end=23)
    assert np.array_equal(whole, part)


@pytest.mark.parametrize("alg", ["222", "333"])
def test_split_oracle_accuracy_improves_with_slices(orc, algs, alg):
    A, B, C = rand(48, 40, 7), rand(40, 52, 8), rand(48, 52, 9)
    ref = orc.fmm_dgemm(algs[alg], A, B, C.copy(order="F"))
    errs = []
    for s in range(2, 9):
        out = orc.split_fmm_dgemm(algs[alg], A, B, C.copy(order="F"), s)
        errs.append(float(np.max(np.abs(out - ref))))
    assert errs[0] < 1e-2
    for a, b in zip(errs, errs[1:4]):
        assert b < a / 16 or b < 1e-15
    assert errs[5] < 1e-13 and errs[6] < 1e-13


@pytest.mark.parametrize("phi", [1.0, 4.0])
def test_split_oracle_hard_inputs(orc, algs, phi):
    """(u - 0.5) * exp(phi * g) inputs: at 7 slices the split form's max-norm
    error against the classical product is within 10x the plain FP64 FMM's."""
    from fmm_blis_gb300 import synth
    A, B = synth.hard(32, 30, 21, phi), synth.hard(30, 34, 22, phi)
    ref = A @ B
    fp64 = orc.fmm_dgemm(algs["222"], A, B, np.zeros((32, 34), order="F"))
    err_fp64 = float(np.max(np.abs(fp64 - ref)))
    out = orc.split_fmm_dgemm(algs["222"], A, B, np.zeros((32, 34), order="F"), 7)
    assert float(np.max(np.abs(out - ref))) <= 10 * err_fp64


def test_split_oracle_zero_and_tiny(orc, algs):
    A = np.zeros((9, 7), order="F")
    B = rand(7, 5, 3)
    C = rand(9, 5, 4)
    out = orc.split_fmm_dgemm(algs["222"], A, B, C.copy(order="F"), 4)
    assert np.array_equal(out, C)
    A = rand(9, 7, 5) * 1e-300
    out = orc.split_fmm_dgemm(algs["222"], A, B, np.zeros((9, 5), order="F"), 7)
    assert np.max(np.abs(out - A @ B)) <= 1e-13 * np.max(np.abs(A @ B)) + 1e-320


def test_split_oracle_fp8_digits(orc, algs):
    """FP8-E4M3 slices (base-32 digits): about 5 bits per slice, the error
    falls with every slice and reaches the FP64 FMM's level at 11-12 slices."""
    rng = np.random.default_rng(41)
    m, n, k = 60, 70, 90
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
    ref = A @ B
    errs = []
    for s in range(3, 13):
        C = np.zeros((m, n), order="F")
        orc.split_fmm_dgemm(algs["222"], A, B, C, s, fmt="fp8")
        errs.append(float(np.abs(C - ref).max()))
    assert all(a > b for a, b in zip(errs[:-3], errs[1:-2]))
    assert errs[-1] < 1e-13
    # s = 6 BF16 (48 bits) and s = 10 FP8 (50 bits) are of the same order
    C = np.zeros((m, n), order="F")
    orc.split_fmm_dgemm(algs["222"], A, B, C, 6)
    e_bf16 = float(np.abs(C - ref).max())
    assert errs[10 - 3] < 4 * e_bf16


@pytest.mark.parametrize("alg,levels,shape,s,fmt,ab", [
    ("222", 1, (7, 9, 5), 6, "bf16", (1.0, 1.0)),
    ("222", 1, (13, 11, 17), 3, "bf16", (-0.75, 0.5)),
    ("232", 1, (9, 10, 8), 8, "bf16", (1.0, 0.0)),
    ("333", 1, (10, 8, 11), 2, "bf16", (2.0, 1.0)),
    ("222", 2, (9, 10, 11), 6, "bf16", (1.0, 1.0)),
    ("222", 1, (6, 5, 300), 6, "bf16", (1.0, 1.0)),     # k_pad > 128: Z in units of level 6
    ("222", 1, (7, 9, 5), 9, "fp8", (1.0, 1.0)),
    ("322", 1, (11, 7, 9), 12, "fp8", (0.5, -1.0)),
    ("222", 1, (8, 6, 40), 4, "fp8", (1.0, 1.0)),
])
def test_split_oracle_equals_independent_restatement(orc, algs, alg, levels, shape, s, fmt, ab):
    """The C oracle's split form equals, bit for bit, a second restatement in
    exact arithmetic written from the definitions (tests/split_restatement.py)."""
    from oracle import coeffs as oc
    from split_restatement import split_fmm
    m, n, k = shape
    a = oc.power(algs[alg], levels)
    A, B, C = rand(m, k, 61 + m), rand(k, n, 62 + n), rand(m, n, 63 + k)
    alpha, beta = ab
    want = split_fmm(a, A, B, C, s, alpha, beta, fmt)
    got = orc.split_fmm_dgemm(a, A, B, C.copy(order="F"), s, alpha, beta, fmt=fmt)
    assert np.array_equal(got, want), float(np.max(np.abs(got - want)))


def test_split_restatement_wide_range_inputs(orc, algs):
    """Entries spread over many binades (digits of small entries far below
    their row's maximum) and exact zeros: still bit for bit."""
    from split_restatement import split_fmm
    rng = np.random.default_rng(5)
    A = np.asfortranarray(rng.uniform(-1, 1, (9, 12)) * np.exp2(rng.integers(-40, 10, (9, 12))))
    B = np.asfortranarray(rng.uniform(-1, 1, (12, 7)) * np.exp2(rng.integers(-30, 30, (12, 7))))
    A[2, :] = 0.0
    B[:, 3] = 0.0
    C = np.asfortranarray(rng.uniform(-1, 1, (9, 7)))
    for fmt, s in (("bf16", 5), ("fp8", 10)):
        want = split_fmm(algs["222"], A, B, C, s, 1.0, 1.0, fmt)
        got = orc.split_fmm_dgemm(algs["222"], A, B, C.copy(order="F"), s, fmt=fmt)
        assert np.array_equal(got, want)


@pytest.mark.parametrize("alg,levels,shape,s,fmt", [("222", 2, (130, 95, 77), 6, "bf16"),
                                                    ("333", 1, (100, 64, 81), 5, "bf16"),
                                                    ("444", 1, (70, 90, 66), 10, "fp8")])
def test_split_rows_mode_equals_full(orc, algs, alg, levels, shape, s, fmt):
    """The oracle's row-subset mode (used to check the GPU at sizes where the
    full restatement would take too long) gives the listed rows exactly the
    full call's bits and touches no other row beyond beta's scaling."""
    from oracle import coeffs as oc
    m, n, k = shape
    a = oc.power(algs[alg], levels)
    A, B, C = rand(m, k, 71), rand(k, n, 72), rand(m, n, 73)
    full = orc.split_fmm_dgemm(a, A, B, C.copy(order="F"), s, alpha=0.75, beta=1.5, fmt=fmt)
    me = -(-m // a[0])
    local = [0, me // 2, me - 1]
    part = orc.split_fmm_dgemm_rows(a, A, B, C.copy(order="F"), s, local, alpha=0.75, beta=1.5, fmt=fmt)
    rows = sorted({r for i in local for r in orc.part_rows(m, a[0], i)})
    assert rows and np.array_equal(part[rows], full[rows])
    other = np.setdiff1d(np.arange(m), rows)
    assert np.array_equal(part[other], 1.5 * C[other])
