"""Loads the reference's own outputs (tests/golden/ref/, written by
tests/golden/make_ref_fixtures.py from bli_strassen_ab_ex, frame/base/
bli_strassen_ab.c:123) and regenerates each case's seeded operands."""
import hashlib
import json

import numpy as np

from conftest import COEFFS, GOLDEN, rand

REF = GOLDEN / "ref"
MANIFEST = json.loads((REF / "manifest.json").read_text())
FULL = sorted(c for c, m in MANIFEST.items() if m["stored"] == "full C_ref")
SAMPLED = sorted(c for c, m in MANIFEST.items() if m["stored"] != "full C_ref")


def case(name):
    """(meta, A, B, C0, stored arrays) of one fixture."""
    meta = MANIFEST[name]
    m, k, n = meta["m"], meta["k"], meta["n"]
    A, B, C = rand(m, k, meta["seed_a"]), rand(k, n, meta["seed_b"]), rand(m, n, meta["seed_c"])
    return meta, A, B, C, np.load(REF / f"{name}.npz")


def alg_of(meta):
    from oracle import coeffs as oc
    return oc.power(oc.read(COEFFS / f"{meta['alg']}.txt"), meta["levels"])


def sha_ok(meta, C_ref):
    return hashlib.sha256(np.asfortranarray(C_ref).tobytes(order="F")).hexdigest() == meta["sha256"]
