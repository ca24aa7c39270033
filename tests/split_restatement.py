"""A second, independent restatement of the split-precision form, in exact
arithmetic, used only to check the C oracle (oracle/fmm_oracle.c) bit for
bit on small shapes.

It follows the definitions rather than the C code's structure: every FP64
rounding point (the operand sums, the bounds, the C updates) is computed
exactly with fractions and rounded once to the nearest double; the digits,
level sums and the fixed-point accumulator Z are Python integers (no int64
wrap-around, so an overflow in the C oracle would show as a mismatch).

Definitions (partition geometry as in frame/base/bli_strassen_ab.c:86-121:
the first d % t parts of a dimension d split t ways get one extra element):

- S_r[i,p] = sum over A sub-blocks q in order of U[q,r] * A_q[i,p] (zero
  outside the sub-block), the first term c * v rounded, each later term as
  one fused multiply-add: round(c * v + sum).
- the row bound b_i = sum over the same q of |U[q,r]| * max_c |A_q[i,c]| in
  the same fused order; E_i = the e with 2^(e-1) <= b_i < 2^e (0 when b_i is
  0); likewise T_r, F_j by columns of B.
- digits of x relative to 2^E, db bits each, s of them: X = x * 2^(db*s-E-1)
  rounded half away from zero, then the balanced digits from the bottom,
  each in [-2^(db-1), 2^(db-1)), the remainder the top digit d_0.
- level g = 2 .. s+1: L_g = sum over slice pairs t + u = g of the digit
  matrix products; Z = sum_{g <= G} L_g 2^(db(G-g)) + sum_{g > G}
  floor(L_g / 2^(db(g-G)) + 1/2), G = 6 for BF16 digits (7 when the k extent
  padded to 64 is at most 128) and min(s+1, 10) for FP8 digits.
- M_r[i,j] = double(Z[i,j]) * 2^(E_i + F_j + 2 - db*G), and every C element
  of sub-block p takes c = round(alpha*W[p,r] * M_r + c) for r in order.
"""
from fractions import Fraction
import math

import numpy as np


def part(d: int, t: int, i: int) -> tuple[int, int]:
    base, rem = divmod(d, t)
    return i * base + min(i, rem), base + (1 if i < rem else 0)


def fused(a: float, b: float, c: float) -> float:
    """round(a * b + c) with one rounding."""
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def exp_above(b: float) -> int:
    return 0 if b == 0.0 else math.frexp(b)[1]


def digits(x: float, E: int, s: int, db: int) -> list[int]:
    v = Fraction(x) * Fraction(2) ** (db * s - E - 1)
    a = abs(v)
    X = int(a + Fraction(1, 2))          # floor(|v| + 1/2): half away from zero
    if v < 0:
        X = -X
    half, base = 1 << (db - 1), 1 << db
    out = [0] * s
    for t in range(s - 1, 0, -1):
        d = (X + half) % base - half
        out[t] = d
        X = (X - d) // base
    out[0] = X
    return out


def split_fmm(alg, A, B, C, s: int, alpha: float = 1.0, beta: float = 1.0, fmt: str = "bf16"):
    mt, kt, nt, R, U, V, W = alg
    A = np.asarray(A, dtype=np.float64)
    B = np.asarray(B, dtype=np.float64)
    C = np.array(C, dtype=np.float64, order="F")
    m, k = A.shape
    n = B.shape[1]
    if beta != 1.0:
        C = np.zeros_like(C) if beta == 0.0 else beta * C
    if m == 0 or n == 0 or k == 0 or alpha == 0.0:
        return C
    db = 5 if fmt == "fp8" else 8
    me, ke, ne = -(-m // mt), -(-k // kt), -(-n // nt)
    k_pad = -(-ke // 64) * 64
    G = min(s + 1, 10) if fmt == "fp8" else (7 if k_pad <= 128 else 6)
    a_rows = [part(m, mt, x) for x in range(mt)]
    k_parts = [part(k, kt, x) for x in range(kt)]
    b_cols = [part(n, nt, x) for x in range(nt)]
    amax = [[max((abs(float(A[i, co + c])) for c in range(cl)), default=0.0) for i in range(m)]
            for (co, cl) in k_parts]
    bmax = [[max((abs(float(B[ro + p, j])) for p in range(rl)), default=0.0) for j in range(n)]
            for (ro, rl) in k_parts]
    Cl = [[float(C[i, j]) for j in range(n)] for i in range(m)]
    for r in range(R):
        if not any(int(W[p, r]) for p in range(mt * nt)):
            continue
        uq = [(q, int(U[q, r])) for q in range(mt * kt) if int(U[q, r])]
        vq = [(q, int(V[q, r])) for q in range(kt * nt) if int(V[q, r])]
        E, F = [], []
        for i in range(me):
            bnd, first = 0.0, True
            for q, c in uq:
                ro, rl = a_rows[q // kt]
                if i >= rl:
                    continue
                mx = amax[q % kt][ro + i]
                bnd = float(abs(c)) * mx if first else fused(float(abs(c)), mx, bnd)
                first = False
            E.append(exp_above(bnd))
        for j in range(ne):
            bnd, first = 0.0, True
            for q, c in vq:
                co, cl = b_cols[q % nt]
                if j >= cl:
                    continue
                mx = bmax[q // nt][co + j]
                bnd = float(abs(c)) * mx if first else fused(float(abs(c)), mx, bnd)
                first = False
            F.append(exp_above(bnd))

        def s_elem(i, p):
            acc, first = 0.0, True
            for q, c in uq:
                ro, rl = a_rows[q // kt]
                co, cl = k_parts[q % kt]
                v = float(A[ro + i, co + p]) if (i < rl and p < cl) else 0.0
                acc = float(c) * v if first else fused(float(c), v, acc)
                first = False
            return acc

        def t_elem(p, j):
            acc, first = 0.0, True
            for q, c in vq:
                ro, rl = k_parts[q // nt]
                co, cl = b_cols[q % nt]
                v = float(B[ro + p, co + j]) if (p < rl and j < cl) else 0.0
                acc = float(c) * v if first else fused(float(c), v, acc)
                first = False
            return acc

        DA = [[digits(s_elem(i, p), E[i], s, db) for p in range(ke)] for i in range(me)]   # [i][p][t]
        DB = [[digits(t_elem(p, j), F[j], s, db) for j in range(ne)] for p in range(ke)]   # [p][j][u]
        M = [[0.0] * ne for _ in range(me)]
        for i in range(me):
            for j in range(ne):
                Z = 0
                for g in range(2, s + 2):
                    L = 0
                    for t in range(1, s + 1):
                        u = g - t
                        if 1 <= u <= s:
                            L += sum(DA[i][p][t - 1] * DB[p][j][u - 1] for p in range(ke))
                    if g <= G:
                        Z += L * (1 << (db * (G - g)))
                    else:
                        sh = db * (g - G)
                        Z += (L + (1 << (sh - 1))) >> sh
                M[i][j] = math.ldexp(float(Z), E[i] + F[j] + 2 - db * G)
        for p in range(mt * nt):
            w = int(W[p, r])
            if not w:
                continue
            ro, rl = a_rows[p // nt]
            co, cl = b_cols[p % nt]
            lam = alpha * float(w)
            for i in range(rl):
                for j in range(cl):
                    Cl[ro + i][co + j] = fused(lam, M[i][j], Cl[ro + i][co + j])
    return np.asfortranarray(np.array(Cl, dtype=np.float64).reshape(m, n))
