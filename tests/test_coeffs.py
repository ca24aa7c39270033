"""Coefficient reader, Brent validator and Kronecker generator of the C ABI
(frame/base/bli_read_fmm.c:24-86 and the reference's coefficient files)."""
import ctypes
import hashlib
import json

import numpy as np
import pytest

from conftest import ALGS, COEFFS, GOLDEN


def test_fixtures_match_manifest():
    man = json.loads((GOLDEN / "manifest.json").read_text())
    for a in ALGS:
        assert hashlib.sha256((COEFFS / f"{a}.txt").read_bytes()).hexdigest() == man[a]["sha256"]
        assert man[a]["brent_violations"] == 0


@pytest.mark.parametrize("name", ALGS)
def test_reader_matches_python_restatement(fmm, algs, name):
    f = fmm.new_fmm(COEFFS / f"{name}.txt")
    try:
        mt, kt, nt, R, U, V, W = algs[name]
        assert (f.m_tilde, f.k_tilde, f.n_tilde, f.R) == (mt, kt, nt, R)
        Uc, Vc, Wc = f.coeffs()
        assert np.array_equal(np.array(Uc), U)
        assert np.array_equal(np.array(Vc), V)
        assert np.array_equal(np.array(Wc), W)
        assert fmm.check_brent(f) == 0
    finally:
        fmm.free_fmm(f)


def test_header_order_is_m_k_n(fmm):
    # 232.txt has m~k~ = 6 rows of U and m~n~ = 4 rows of W: header is m~ k~ n~ R
    f = fmm.new_fmm(COEFFS / "232.txt")
    try:
        assert (f.m_tilde, f.k_tilde, f.n_tilde, f.R) == (2, 3, 2, 11)
    finally:
        fmm.free_fmm(f)


def test_long_lines(fmm):
    # 444.txt rows are longer than the reference's 128-byte line buffer
    assert max(len(l) for l in open(COEFFS / "444.txt")) > 128
    f = fmm.new_fmm(COEFFS / "444.txt")
    try:
        assert f.R == 49 and fmm.check_brent(f) == 0
    finally:
        fmm.free_fmm(f)


def test_strassen_builtin_equals_222(fmm, algs):
    s = fmm.strassen_fmm()
    mt, kt, nt, R, U, V, W = algs["222"]
    Uc, Vc, Wc = s.coeffs()
    assert np.array_equal(np.array(Uc), U) and np.array_equal(np.array(Vc), V) and np.array_equal(np.array(Wc), W)


def test_missing_and_malformed_files(fmm, tmp_path):
    with pytest.raises(fmm.FmmError) as e:
        fmm.new_fmm(tmp_path / "nope.txt")
    assert e.value.status == 2
    bad = tmp_path / "bad.txt"
    bad.write_text("2 2 2 7\n1 0 1\n")
    with pytest.raises(fmm.FmmError) as e:
        fmm.new_fmm(bad)
    assert e.value.status == 3
    short = tmp_path / "short.txt"
    short.write_text("2 2 2 7\n" + "1 0 1 0 1 -1 0\n" * 5)
    with pytest.raises(fmm.FmmError) as e:
        fmm.new_fmm(short)
    assert e.value.status == 3
    # the by-value reader keeps the reference signature and returns R == 0
    f = fmm.lib().new_fmm(str(tmp_path / "nope.txt").encode())
    assert f.R == 0 and not f.U


def test_wrong_coefficients_fail_brent(fmm, tmp_path):
    txt = (COEFFS / "222.txt").read_text().replace("1 0 1 0 1 -1 0", "1 0 1 0 1 1 0", 1)
    p = tmp_path / "wrong.txt"
    p.write_text(txt)
    f = fmm.new_fmm(p)
    try:
        assert fmm.check_brent(f) > 0
    finally:
        fmm.free_fmm(f)


@pytest.mark.parametrize("outer,inner", [("222", "222"), ("232", "322"), ("333", "222")])
def test_kron_is_valid_and_matches_restatement(fmm, algs, outer, inner):
    from oracle import coeffs as oc
    fo = fmm.new_fmm(COEFFS / f"{outer}.txt")
    fi = fmm.new_fmm(COEFFS / f"{inner}.txt")
    k = fmm.kron(fo, fi)
    try:
        ref = oc.kron(algs[outer], algs[inner])
        assert (k.m_tilde, k.k_tilde, k.n_tilde, k.R) == ref[:4]
        Uc, Vc, Wc = k.coeffs()
        assert np.array_equal(np.array(Uc), ref[4])
        assert np.array_equal(np.array(Vc), ref[5])
        assert np.array_equal(np.array(Wc), ref[6])
        assert fmm.check_brent(k) == 0
    finally:
        fmm.free_fmm(k)
        fmm.free_fmm(fo)
        fmm.free_fmm(fi)


def test_bl_clock_monotonic(fmm):
    a = fmm.bl_clock()
    b = fmm.bl_clock()
    assert b >= a >= 0.0


def test_package_ships_the_reference_coefficient_files():
    """The algorithms the package and its tuner load (fmm_blis_gb300/coeffs/)
    are the reference's files byte for byte (the pinned fixtures)."""
    import hashlib
    import json
    from conftest import ROOT
    man = json.loads((GOLDEN / "manifest.json").read_text())
    for a in ALGS:
        data = (ROOT / "fmm_blis_gb300" / "coeffs" / f"{a}.txt").read_bytes()
        assert hashlib.sha256(data).hexdigest() == man[a]["sha256"]
