"""Per-problem plan choice for the FMM GEMM: form, algorithm, recursion depth,
slice count.

The reference fixes the algorithm (the coefficient file handed to
bli_strassen_ab_ex, frame/base/bli_strassen_ab.c:123) and runs one recursion
level; it has no tuner. For batched and served mixes of uneven shapes this
module picks, per problem, among classical (levels 0) and the coefficient
files at one or two levels, by a cost model of the GB300 kernels of this
library, and, for the split form, the fewest BF16 slices whose predicted error
meets the requested relative error.

Cost model (calibrated on GB300 at m = n = k = 16384, SM clock 1.8-2.07 GHz):
  FP64 form: a CTA per 64 x 64 tile position of the product grid runs all
    R products over it, the CTAs of an SM share its FP64 pipe (2 FMA/clk):
    time = ceil(tiles / SMs) * 2048 * k_e * R / clock / 0.98, plus, for FMM
    algorithms, one HBM write and read of every product's operand
    combinations (formed once ahead of the tiles). (16384^3: classical
    7.03 s measured, 7.14 s modelled; 444 two levels 5.24 / 4.96 s;
    333 two levels 5.86 / 5.55 s.) Grids too small to fill the SMs use
    32 x 32 tiles; classical problems with a small output and a long k take
    the small/skinny path (clusters of CTAs splitting k; 128 x 128 x 16384:
    1.05 ms measured, 1.01 ms modelled).
  Split form: the persistent tcgen05 GEMM runs (problem, product, 128 x 256
    tile) items on 152 CTAs, each item s(s+1)/2 slice pairs x k_pad/64 blocks
    of 512 MMA clocks at about 61% of 2.07 GHz under the power cap
    (222 two levels, 6 slices: 90 ms modelled, 84-87 ms measured for the
    single call; refitting to 65% moved large served requests to plans that
    measured a p99 of 431 ms against 37 ms in a 30 s stream at 200/s, so the
    batched path that serves them is what the constant follows); the digit packs cost 1.16 ps
    per element-slice and side, the multi-C scatter 2.44 ps per W entry and
    element, the row/column maxima one read of A and B.

Input-aware slice choice (Tuner.plan_for): the model above assumes inputs
whose entries are of one magnitude. For wider-range inputs (config 3's
(u - 0.5) exp(phi g) with phi = 1, 4) the per-row and per-column power-of-two
scales lose the low bits of entries far below their row's or column's
maximum, and the error per slice falls more slowly. plan_for measures the
error on a sample of the problem itself -- the 128 rows of A and columns of B
with the largest maxima plus 128 evenly spread ones, all of k -- split with
the plan's slice count at levels 0 against the FP64 classical product of the
sample; a row's exponent depends only on its own maxima, so the sampled rows
and columns get exactly the digits the full call gives them. The slice count
grows until the sample's error, times the FMM level growth and the safety
factor, meets the target.

Error model (split form, uniform-like inputs): the max-norm error relative to
max|C| of s slices of db-bit digits is about 0.4 * 2^(-db*s) * sqrt(k) *
1.5^levels (222 two levels, k = 16384: 6 BF16 slices 1.6e-13 measured, 4.1e-13
modelled; 10 FP8 slices 5.8e-14 / 1.0e-13). The tuner keeps a safety factor
of 4 on it. FP8-E4M3 slices (db = 5) run a slice pair at twice the BF16 rate
but at about 10% lower SM clock under the power cap (GEMM 2788 vs 1477
TFLOP/s executed at 1.67 vs 1.83 GHz): a pair costs 0.55 of a BF16 pair.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from pathlib import Path

COEFF_DIR = Path(__file__).resolve().parent / "coeffs"   # the algorithms shipped with the package

SMS = 152
CLOCK_HZ = 2.07e9
FP64_EFF = 0.98
FP64_SMALL_EFF = 0.8      # 32 x 32 tiles (two CTAs per SM)
FP64_SUP_EFF = 0.5        # small/skinny cluster CTAs, up to two per SM: 128 x 128 x 16384 in 1.05 ms
SPLIT_EFF = 0.61
PACK_S_PER_ELEM_SLICE = 1.16e-12
SCATTER_S_PER_ENTRY_ELEM = 2.44e-12
HBM_BPS = 6.0e12
LAUNCH_S = 4e-6
ERR_C0 = 0.4
ERR_LEVEL_GROWTH = 1.5
ERR_SAFETY = 4.0
FP8_PAIR_COST = 0.55
DIGIT_BITS = {"bf16": 8, "fp8": 5}
SLICE_RANGE = {"bf16": (3, 8), "fp8": (3, 12)}


def _sup_splits(m: int, n: int, k: int) -> int:
    """k chunks of the library's small/skinny classical FP64 path (0: the
    regular kernel); a host-only query of the shape rule."""
    from . import f64_sup_splits
    return f64_sup_splits(m, n, k)


def _cdiv(a: int, b: int) -> int:
    return -(-a // b)


def _round_up(a: int, b: int) -> int:
    return _cdiv(a, b) * b


@dataclass(frozen=True)
class AlgShape:
    """What the cost model needs of a (flattened) algorithm."""

    name: str            # coefficient file stem, "classical" for the plain GEMM
    levels: int
    mt: int
    kt: int
    nt: int
    R: int
    nnz_u: float         # average nonzeros per product column of U
    nnz_v: float
    nnz_w: int           # total nonzeros of W


def alg_shapes(names=("222", "232", "322", "333", "444"), levels=(1, 2)) -> list[AlgShape]:
    """Classical plus every coefficient file at the given recursion levels,
    read with the library's own reader (new_fmm, the format of
    frame/base/bli_read_fmm.c:24-86)."""
    from . import free_fmm, new_fmm

    out = [AlgShape("classical", 0, 1, 1, 1, 1, 1.0, 1.0, 1)]
    for nm in names:
        f = new_fmm(COEFF_DIR / f"{nm}.txt")
        try:
            U, V, W = f.coeffs()
            mt, kt, nt, R = f.m_tilde, f.k_tilde, f.n_tilde, f.R
        finally:
            free_fmm(f)
        nu = [sum(1 for row in U if row[r] != 0) for r in range(R)]
        nv = [sum(1 for row in V if row[r] != 0) for r in range(R)]
        nw = sum(1 for row in W for x in row if x != 0)
        for L in levels:
            out.append(AlgShape(nm, L, mt ** L, kt ** L, nt ** L, R ** L,
                                (sum(nu) / R) ** L, (sum(nv) / R) ** L, nw ** L))
    return out


@dataclass
class Plan:
    form: str                  # "fp64" or "split"
    alg: str                   # coefficient file stem or "classical"
    levels: int
    slices: int                # 0 for the FP64 form
    est_s: float               # modelled device time
    est_rel_err: float | None  # modelled max-norm error / max|C| (split form)
    fmt: str = "bf16"          # slice format of the split form: "bf16" or "fp8"
    candidates: list = field(default_factory=list, repr=False)


def fp64_time(a: AlgShape, m: int, n: int, k: int) -> float:
    me, ne, ke = _cdiv(m, a.mt), _cdiv(n, a.nt), _cdiv(k, a.kt)
    tiles = _cdiv(me, 64) * _cdiv(ne, 64)
    per_sm = _cdiv(tiles, SMS)
    gemm = per_sm * 2048.0 * ke * a.R / CLOCK_HZ / FP64_EFF
    # grids too small to fill the SMs take 32 x 32 tiles, two CTAs per SM
    gemm = min(gemm, _cdiv(_cdiv(me, 32) * _cdiv(ne, 32), 2 * SMS) * 1024.0 * ke * a.R / CLOCK_HZ / FP64_SMALL_EFF)
    if a.R == 1:
        ks = _sup_splits(m, n, k)
        if ks:
            # small/skinny classical path: clusters of ks CTAs, one per k chunk
            kc = _round_up(_cdiv(k, ks), 32)
            ctas = _cdiv(m, 32) * _cdiv(n, 32) * ks
            return _cdiv(ctas, 2 * SMS) * 512.0 * kc / CLOCK_HZ / FP64_SUP_EFF + 2 * LAUNCH_S
        return gemm + 2 * LAUNCH_S
    # FMM: each product's operand combinations are formed once ahead of the
    # tiles (written, then read back: HBM), so the tiles see single-term operands
    combine = a.R * (me * ke + ke * ne) * 8.0 * 2.0 / HBM_BPS
    return gemm + combine + 4 * LAUNCH_S


def split_time(a: AlgShape, m: int, n: int, k: int, s: int, fmt: str = "bf16") -> float:
    me, ne, ke = _cdiv(m, a.mt), _cdiv(n, a.nt), _cdiv(k, a.kt)
    kbe = 128 if fmt == "fp8" else 64        # k elements per 128-byte stage row
    m_pad, n_pad, k_pad = _round_up(max(me, 1), 128), _round_up(max(ne, 1), 256), _round_up(max(ke, 1), kbe)
    items = a.R * (m_pad // 128) * (n_pad // 256)
    waves = _cdiv(items, SMS)
    pairs = s * (s + 1) // 2
    gemm = waves * pairs * (k_pad // 64) * 512.0 / (CLOCK_HZ * SPLIT_EFF)
    if fmt == "fp8":
        gemm *= FP8_PAIR_COST
    pack = a.R * (m_pad + n_pad) * k_pad * s * PACK_S_PER_ELEM_SLICE
    scatter = a.nnz_w * me * ne * SCATTER_S_PER_ENTRY_ELEM
    maxima = 8.0 * (m * k + k * n) / HBM_BPS
    return gemm + pack + scatter + maxima + 7 * LAUNCH_S


def split_rel_err(a: AlgShape, k: int, s: int, fmt: str = "bf16") -> float:
    return ERR_C0 * 2.0 ** (-DIGIT_BITS[fmt] * s) * math.sqrt(max(k, 1)) * ERR_LEVEL_GROWTH ** a.levels


def _fits(a: AlgShape, m: int, n: int, k: int, min_block: int) -> bool:
    """FMM levels only where every sub-block keeps a useful size."""
    if a.levels == 0:
        return True
    return min(_cdiv(m, a.mt), _cdiv(n, a.nt), _cdiv(k, a.kt)) >= min_block


class Tuner:
    """Chooses a Plan per (m, n, k, form, target error). Deterministic: the
    same request always gets the same plan, so a result served in a mix is the
    one served alone."""

    def __init__(self, algs: list[AlgShape] | None = None, min_block_fp64: int = 256,
                 min_block_split: int = 1024, formats=("bf16", "fp8")):
        self.algs = algs if algs is not None else alg_shapes()
        self.min_block_fp64 = min_block_fp64
        self.min_block_split = min_block_split
        self.formats = tuple(formats)
        self.cache: dict = {}

    def plan(self, m: int, n: int, k: int, form: str = "split", target_rel_err: float = 1e-10) -> Plan:
        key = (m, n, k, form, target_rel_err)
        if key in self.cache:
            return self.cache[key]
        cands = []
        for a in self.algs:
            if form == "fp64":
                if not _fits(a, m, n, k, self.min_block_fp64):
                    continue
                cands.append(Plan("fp64", a.name, a.levels, 0, fp64_time(a, m, n, k), None))
            else:
                if not _fits(a, m, n, k, self.min_block_split):
                    continue
                for fmt in self.formats:
                    lo, hi = SLICE_RANGE[fmt]
                    for s in range(lo, hi + 1):
                        err = split_rel_err(a, k, s, fmt)
                        if err * ERR_SAFETY <= target_rel_err:
                            cands.append(Plan("split", a.name, a.levels, s, split_time(a, m, n, k, s, fmt), err, fmt))
                            break
        if not cands:
            raise ValueError(f"no plan meets the target for m={m} n={n} k={k} form={form} "
                             f"target={target_rel_err}")
        cands.sort(key=lambda p: p.est_s)
        best = cands[0]
        best.candidates = cands
        self.cache[key] = best
        return best

    def plan_for(self, fmm, A, B, target_rel_err: float = 1e-10) -> Plan:
        """Split-form plan for these operands (column-major CUDA tensors): the
        shape plan, with slices added while a measured sample of the problem
        (sample_rel_err, times the FMM level growth and the safety factor)
        misses the target. Deterministic for given operands; not cached (it
        depends on the data)."""
        m, k = A.shape
        n = B.shape[1]
        base = self.plan(m, n, k, "split", target_rel_err)
        hi = SLICE_RANGE[base.fmt][1]
        growth = ERR_LEVEL_GROWTH ** base.levels
        s = base.slices
        while True:
            err = sample_rel_err(fmm, A, B, s, base.fmt) * growth
            if err * ERR_SAFETY <= target_rel_err or s >= hi:
                break
            s += 1
        if s == base.slices:
            return base
        a = next(x for x in self.algs if x.name == base.alg and x.levels == base.levels)
        return Plan("split", base.alg, base.levels, s, split_time(a, m, n, k, s, base.fmt), err, base.fmt)


def sample_rel_err(fmm, A, B, slices: int, fmt: str = "bf16", count: int = 128) -> float:
    """Max-norm error relative to max|C| of the levels-0 split form on a
    sample of the product A*B (column-major CUDA tensors): the `count` rows of
    A and columns of B with the largest maxima plus `count` evenly spread
    ones, all of k, against the FP64 classical product of the same sample.
    The sampled rows and columns keep their exponents (they depend on the
    row's or column's own maxima only), so their digits are the full call's."""
    import torch

    m, k = A.shape
    n = B.shape[1]

    def pick(mx, d):
        top = torch.topk(mx, min(count, d)).indices
        spread = torch.linspace(0, d - 1, min(count, d), device=mx.device).round().long()
        return torch.unique(torch.cat([top, spread]))

    rows = pick(A.abs().amax(dim=1), m)
    cols = pick(B.abs().amax(dim=0), n)
    As = A[rows].t().contiguous().t()           # column-major copies of the sample
    Bs = B[:, cols].t().contiguous().t()
    Cs = torch.zeros((len(cols), len(rows)), dtype=torch.float64, device=A.device).t()
    Cr = torch.zeros_like(Cs.t()).t()
    fmm.split_dgemm(As, Bs, Cs, None, 0, slices, fmt=fmt)
    fmm.dgemm(As, Bs, Cr, None, 0)
    ref = float(Cr.abs().max())
    return float((Cs - Cr).abs().max()) / ref if ref > 0 else 0.0
