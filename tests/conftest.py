import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
COEFFS = GOLDEN / "coeffs"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

ALGS = ["222", "232", "322", "333", "444"]

# c of the plain FP64 form's normwise bound |C - C_other| <= c * eps64 * k * max|A| * max|B| (+ 4 eps max|C0|),
# per (algorithm, levels): the same bound holds between this library's GPU FP64 form, the oracle and the
# reference's own bli_strassen_ab_ex (tests/golden/ref/), which differ only in the order of their k-sums.
C_BOUND = {("222", 1): 4, ("232", 1): 4, ("322", 1): 4, ("333", 1): 8, ("444", 1): 8,
           ("222", 2): 8, ("232", 2): 8, ("322", 2): 8, ("333", 2): 16, ("444", 2): 16}


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); run with -m gpu")


@pytest.fixture(scope="session")
def fmm():
    """The product library (built in-tree if needed)."""
    from fmm_blis_gb300 import build
    build.build()
    import fmm_blis_gb300
    fmm_blis_gb300.lib()
    return fmm_blis_gb300


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def algs():
    from oracle import coeffs as oc
    return {a: oc.read(COEFFS / f"{a}.txt") for a in ALGS}


def rand(m, n, seed):
    from fmm_blis_gb300 import synth
    return synth.uniform(m, n, seed)


def fmm_bound(A, B, C0, k, c):
    """c * eps64 * k * max|A| * max|B| (+ rounding of C's own magnitude)."""
    eps = np.finfo(np.float64).eps
    amax = float(np.max(np.abs(A))) if A.size else 0.0
    bmax = float(np.max(np.abs(B))) if B.size else 0.0
    cmax = float(np.max(np.abs(C0))) if C0.size else 0.0
    return c * eps * max(k, 1) * amax * bmax + 4 * eps * cmax
