"""Regenerates tests/golden/ from the reference checkout (run in the build
container, where the reference is mounted; the GPU machine only reads the
committed outputs).

coeffs/*.txt   the reference's coefficient files 222, 232, 322, 333, 444,
               byte for byte (they define the algorithms and their format is
               part of the drop-in contract); manifest.json records their
               sha256, header and Brent-equation check.
kat_3x13x7.npz the reference's one known-answer case (test/test_strassen_oapi.c:
               252, m=3 n=13 k=7, C := C + A*B) on seeded inputs, with the
               exact product computed in rational arithmetic and rounded once
               to float64, so any correct FP64 FMM lands within a few ulps.
exact_*.npz    the same for a few uneven shapes used by the parity tests.
"""
from __future__ import annotations

import hashlib
import json
import shutil
import sys
from fractions import Fraction
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))

from fmm_blis_gb300 import synth  # noqa: E402
from oracle import coeffs as oc  # noqa: E402

REF = Path("/root/reference")
FILES = ["222", "232", "322", "333", "444"]


def exact_update(A, B, C):
    m, k = A.shape
    n = B.shape[1]
    out = np.empty_like(C)
    for i in range(m):
        for j in range(n):
            s = Fraction(float(C[i, j]))
            for p in range(k):
                s += Fraction(float(A[i, p])) * Fraction(float(B[p, j]))
            out[i, j] = float(s)
    return np.asfortranarray(out)


def main() -> None:
    (HERE / "coeffs").mkdir(exist_ok=True)
    manifest = {}
    for f in FILES:
        src = REF / f"{f}.txt"
        dst = HERE / "coeffs" / f"{f}.txt"
        shutil.copyfile(src, dst)
        alg = oc.read(dst)
        manifest[f] = {
            "sha256": hashlib.sha256(dst.read_bytes()).hexdigest(),
            "header_mkn_R": list(alg[:4]),
            "brent_violations": oc.brent_violations(alg),
        }
    (HERE / "manifest.json").write_text(json.dumps(manifest, indent=1) + "\n")
    for name, (m, n, k, seed) in {"kat_3x13x7": (3, 13, 7, 1), "exact_17x9x23": (17, 9, 23, 2),
                                  "exact_33x31x40": (33, 31, 40, 3)}.items():
        A = synth.uniform(m, k, seed)
        B = synth.uniform(k, n, seed + 100)
        C = synth.uniform(m, n, seed + 200)
        np.savez(HERE / f"{name}.npz", A=A, B=B, C=C, C_out=exact_update(A, B, C), seed=seed)
    print("wrote", HERE)


if __name__ == "__main__":
    main()
