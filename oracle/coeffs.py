"""ORACLE -- test infrastructure only: a plain-Python reader of the U/V/W
coefficient files (frame/base/bli_read_fmm.c:24-80, header in the order the
files are written: m~ k~ n~ R), the Brent equations and the Kronecker
product, used to cross-check the library's C reader."""
from __future__ import annotations

import itertools

import numpy as np


def read(path):
    rows = []
    for line in open(path):
        s = line.strip()
        if not s or s.startswith("#"):
            continue
        rows.append([int(x) for x in s.split()])
    mt, kt, nt, R = rows[0]
    body = rows[1:]
    a, b, c = mt * kt, kt * nt, mt * nt
    assert len(body) == a + b + c, path
    U = np.array(body[:a], dtype=np.int32)
    V = np.array(body[a:a + b], dtype=np.int32)
    W = np.array(body[a + b:], dtype=np.int32)
    assert U.shape[1] == V.shape[1] == W.shape[1] == R
    return (mt, kt, nt, R, U, V, W)


def brent_violations(alg) -> int:
    mt, kt, nt, R, U, V, W = alg
    bad = 0
    for a, b, b2, c, a2, c2 in itertools.product(range(mt), range(kt), range(kt), range(nt), range(mt),
                                                 range(nt)):
        s = int(np.sum(U[a * kt + b].astype(np.int64) * V[b2 * nt + c] * W[a2 * nt + c2]))
        want = int(a == a2 and b == b2 and c == c2)
        bad += s != want
    return bad


def kron(o, i):
    """Flat block (a, b) = inner block (a % ti, b % ti2) of outer block (a // ti, b // ti2)."""
    mo, ko, no, Ro, Uo, Vo, Wo = o
    mi, ki, ni, Ri, Ui, Vi, Wi = i

    def fac(Fo, ro, co, Fi, ri, ci):
        rows, cols = ro * ri, co * ci
        out = np.zeros((rows * cols, Ro * Ri), dtype=np.int32)
        for a in range(rows):
            for b in range(cols):
                qo = (a // ri) * co + b // ci
                qi = (a % ri) * ci + b % ci
                out[a * cols + b] = np.outer(Fo[qo], Fi[qi]).reshape(-1)
        return out

    return (mo * mi, ko * ki, no * ni, Ro * Ri, fac(Uo, mo, ko, Ui, mi, ki), fac(Vo, ko, no, Vi, ki, ni),
            fac(Wo, mo, no, Wi, mi, ni))


def classical():
    one = np.ones((1, 1), dtype=np.int32)
    return (1, 1, 1, 1, one, one, one)


def power(alg, levels):
    if levels == 0:
        return classical()
    out = alg
    for _ in range(levels - 1):
        out = kron(out, alg)
    return out
