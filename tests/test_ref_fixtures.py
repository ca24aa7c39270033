"""The oracle against the reference's own outputs.

tests/golden/ref/ holds C from the reference's bli_strassen_ab_ex
(frame/base/bli_strassen_ab.c:123), built from its sources by
oracle/build_ref.sh and run by tests/golden/make_ref_fixtures.py on seeded
operands with alpha = beta = 1: every coefficient file at one level on the
reference test's shape (m=3, k=7, n=13, test/test_strassen_oapi.c:252), an
uneven 97x61x45 and 256^3; every file at two levels (Kronecker algorithms) on
160x144x176; Strassen at two levels on 256^3; Strassen at one level on
2048^3 (sampled entries). The oracle must agree with each within the plain
FP64 form's normwise bound (conftest.C_BOUND): the two differ only in the
order of their k-sums."""
import numpy as np
import pytest

from conftest import C_BOUND, fmm_bound
from ref_fixtures import FULL, MANIFEST, SAMPLED, alg_of, case, sha_ok


def test_fixture_set_covers_every_algorithm_and_level():
    seen = {(m["alg"], m["levels"]) for m in MANIFEST.values()}
    assert seen == set(C_BOUND)
    assert any(m["build"] == "asis" for m in MANIFEST.values())


@pytest.mark.parametrize("name", FULL)
def test_oracle_matches_reference_output(orc, name):
    meta, A, B, C, z = case(name)
    C_ref = z["C_ref"]
    assert C_ref.shape == C.shape and sha_ok(meta, C_ref)
    got = orc.fmm_dgemm(alg_of(meta), A, B, C.copy(order="F"))
    c = C_BOUND[(meta["alg"], meta["levels"])]
    assert np.max(np.abs(got - C_ref)) <= fmm_bound(A, B, C, meta["k"], c)


@pytest.mark.parametrize("name", SAMPLED)
def test_oracle_matches_reference_output_sampled(orc, name):
    """2048^3 (the size of Strassen's one-level configuration): the oracle on
    the whole problem against the reference's sampled entries and norms."""
    meta, A, B, C, z = case(name)
    got = orc.fmm_dgemm(alg_of(meta), A, B, C.copy(order="F"))
    c = C_BOUND[(meta["alg"], meta["levels"])]
    bound = fmm_bound(A, B, C, meta["k"], c)
    assert np.max(np.abs(got[z["i"], z["j"]] - z["values"])) <= bound
    assert abs(np.linalg.norm(got) - float(z["fro"])) <= bound * np.sqrt(got.size)
    assert abs(got.sum() - float(z["sum"])) <= bound * got.size


def test_reference_fmm_is_not_the_classical_product():
    """The fixtures are FMM outputs, not a classical GEMM's: on 256^3 the
    reference's 444 result differs from the exact-order classical product
    in its last bits (the FMM's own rounding), while staying in its bound."""
    import oracle
    meta, A, B, C, z = case("444x1_256x256x256")
    classical = oracle.dgemm(A, B, C.copy(order="F"))
    assert not np.array_equal(classical, z["C_ref"])
