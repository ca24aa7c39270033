"""Records the reference's own FMM outputs as golden fixtures (tests/golden/ref/).

Runs in the build container, where the reference sources are mounted: it
builds them with oracle/build_ref.sh (into oracle/_ref/, git-ignored), then
for every case below writes seeded operands to oracle/ref_fixture.x, which
calls the reference's bli_strassen_ab_ex (frame/base/bli_strassen_ab.c:123)
with alpha = beta = 1, and keeps the C it returns. The GPU machine and the
tests only read the committed .npz files and regenerate the operands from
their seeds (fmm_blis_gb300.synth.uniform).

Build used per case: "asis" (the reference exactly as shipped) for Strassen
222 at one level, the case it computes correctly; "patched" (the three
one-line fixes listed in oracle/build_ref.sh) for every other algorithm and
for two-level (Kronecker) algorithms. For 222 at one level both builds are
run and must agree bit for bit.

Fixtures:
  ref/<alg>x<L>_<m>x<k>x<n>.npz   C_ref (float64, column-major) and the seeds
  ref/222x1_2048x2048x2048.npz    config-1 size: 8192 sampled entries of C_ref
                                  (seeded positions), plus sum and Frobenius
                                  norm of the whole C_ref
  ref/manifest.json               per case: algorithm, levels, shape, seeds,
                                  build, reference time, sha256 of C_ref
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))

from fmm_blis_gb300 import synth  # noqa: E402
from oracle import coeffs as oc  # noqa: E402

OUT = HERE / "ref"
REF_BUILD = REPO / "oracle" / "_ref"
ALGS = ["222", "232", "322", "333", "444"]
SAMPLES = 8192


def cases():
    out = []
    for a in ALGS:
        out += [(a, 1, 3, 7, 13), (a, 1, 97, 61, 45), (a, 1, 256, 256, 256), (a, 2, 160, 144, 176)]
    out += [("222", 2, 256, 256, 256), ("222", 1, 2048, 2048, 2048)]
    return out


def seeds(m, k, n):
    base = (m * 73856093 ^ k * 19349663 ^ n * 83492791) % 100000
    return base + 1, base + 2, base + 3


def run_ref(variant, alg, A, B, C):
    mt, kt, nt, R, U, V, W = alg
    m, k = A.shape
    n = B.shape[1]
    exe = REF_BUILD / variant / "ref_fixture.x"
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "in.bin", Path(td) / "out.bin"
        with open(fin, "wb") as f:
            np.array([m, n, k, mt, kt, nt, R], dtype=np.int64).tofile(f)
            for X in (U, V, W):
                np.ascontiguousarray(X, dtype=np.int32).tofile(f)
            for X in (A, B, C):
                np.asarray(X, dtype=np.float64).ravel(order="F").tofile(f)
        env = dict(os.environ, BLIS_NUM_THREADS=str(os.cpu_count() or 1))
        p = subprocess.run([str(exe), str(fin), str(fout)], capture_output=True, text=True, env=env)
        if p.returncode != 0:
            raise RuntimeError(f"{exe} failed: {p.stdout}{p.stderr}")
        out = np.fromfile(fout, dtype=np.float64).reshape((n, m)).T
        return np.asfortranarray(out), float(p.stdout.split()[-1])


def main() -> None:
    if not (REF_BUILD / "patched" / "ref_fixture.x").exists() or not (REF_BUILD / "asis" / "ref_fixture.x").exists():
        subprocess.run(["bash", str(REPO / "oracle" / "build_ref.sh")], check=True)
    OUT.mkdir(exist_ok=True)
    manifest = {}
    for name, levels, m, k, n in cases():
        alg = oc.power(oc.read(HERE / "coeffs" / f"{name}.txt"), levels)
        sa, sb, sc = seeds(m, k, n)
        A, B, C = synth.uniform(m, k, sa), synth.uniform(k, n, sb), synth.uniform(m, n, sc)
        variant = "asis" if (name, levels) == ("222", 1) else "patched"
        Cref, t = run_ref(variant, alg, A, B, C)
        if variant == "asis":
            Cp, _ = run_ref("patched", alg, A, B, C)
            assert np.array_equal(Cp, Cref), f"{name}: as-is and patched reference builds differ"
        case = f"{name}x{levels}_{m}x{k}x{n}"
        meta = dict(alg=name, levels=levels, m=m, k=k, n=n, seed_a=sa, seed_b=sb, seed_c=sc, build=variant,
                    ref_seconds=round(t, 4), sha256=hashlib.sha256(Cref.tobytes(order="F")).hexdigest())
        if m * n > 1 << 20:
            rng = np.random.default_rng(sa)
            ii = rng.integers(0, m, SAMPLES)
            jj = rng.integers(0, n, SAMPLES)
            np.savez_compressed(OUT / f"{case}.npz", i=ii, j=jj, values=Cref[ii, jj], sum=Cref.sum(),
                                fro=np.linalg.norm(Cref), seeds=np.array([sa, sb, sc]))
            meta["stored"] = f"{SAMPLES} sampled entries, sum, Frobenius norm"
        else:
            np.savez_compressed(OUT / f"{case}.npz", C_ref=Cref, seeds=np.array([sa, sb, sc]))
            meta["stored"] = "full C_ref"
        manifest[case] = meta
        print(case, variant, f"{t:.3f}s", flush=True)
    (OUT / "manifest.json").write_text(json.dumps(manifest, indent=1) + "\n")


if __name__ == "__main__":
    main()
