/*
 * Split-precision (Ozaki-style) form of the FMM GEMM on the sm_103a tensor
 * cores, with BF16 slices (base-256 digits, tcgen05 kind::f16) or FP8-E4M3
 * slices (base-32 digits, kind::f8f6f4). db below is the digit width: 8 or 5.
 *
 * Per product r of the (flattened) FMM algorithm:
 *
 *   1. exps:   row exponents E_i of S_r = sum_q U[q,r] A_q and column
 *              exponents F_j of T_r = sum_q V[q,r] B_q, from the bound
 *              |S_r[i,:]| <= sum_q |U[q,r]| * max|A_q[i,:]|, evaluated in FP64
 *              in the same order as the sums themselves (so the bound holds
 *              for the rounded sums too). The per-sub-block row/column maxima
 *              are computed once per call (amax/bmax kernels). These
 *              power-of-two scales are per row of S_r and per column of T_r
 *              for both formats: a scale that varied along k would give each
 *              k block's products a different weight and end the exact
 *              integer accumulation over k.
 *   2. pack:   the fused multi-operand pack (plugin/ref_kernels/
 *              bli_packm_fmm_ref.c:89-147): S_r (T_r) is formed in FP64 in
 *              sub-block order with zero fill, then split there into `s`
 *              balanced base-2^db digits d_1..d_s:
 *                  S[i,p] ~= 2^(E_i + 1 - db*s) * sum_t d_t[i,p] 2^(db(s-t))
 *              using integer arithmetic on the FP64 bit pattern. BF16 digits
 *              are integers in [-128, 128] (at most 8 significant bits), FP8
 *              digits integers in [-16, 16] (at most 4): exact either way.
 *              Digits are written K-major ("slices" [t][row][k]).
 *   3. gemm:   tcgen05.mma (FP32 accumulation in TMEM) over the slice pairs
 *              (t,u) with t+u = g for the levels g = 2..s+1. A digit product
 *              is an integer of magnitude <= 2^14 (BF16) or 2^8 (FP8), so a
 *              chunk of 16 stage rows (1024 BF16 or 2048 FP8 terms) sums to an
 *              integer of magnitude <= 2^24 that FP32 holds exactly; the
 *              epilogue warps drain each chunk from TMEM (double-buffered, so
 *              the tensor core keeps running), convert it exactly to int32 and
 *              add it to the level sum L_g. At the end of a level, L_g is
 *              folded into a 64-bit fixed-point accumulator Z in global
 *              memory in units of level G (BF16: G = 6, or 7 when
 *              k_pad <= 128; FP8: G = min(s + 1, 10); the finest units that
 *              keep Z inside int64):
 *                  Z = sum_{g<=G} L_g * 2^(db(G-g)) + sum_{g>G} round(L_g / 2^(db(g-G)))
 *              and M_r[i,j] ~= 2^(E_i + F_j + 2 - db*G) * Z is formed in FP64
 *              and added with alpha*W[p,r] into every C sub-block p (the
 *              multi-C epilogue, plugin/ref_kernels/bli_gemm_fmm_ref.c:99-120).
 *
 * FP64 is only used for the packing sums, the bounds, the int64 -> FP64
 * conversion and the C updates; the digit split, the level sums and Z are
 * exact integer arithmetic, so the result is deterministic and reproducible
 * bit for bit by a CPU restatement.
 *
 * Limits: k_e = ceil(k/k~) <= 16384 per call (level sums stay inside int32
 * and Z inside int64); slices 2..8 (BF16) or 2..12 (FP8); finite inputs.
 *
 * Execution. Two persistent GEMM kernels: split_gemm_kernel (one CTA per SM,
 * 128 x 256 tiles) and split_gemm_pair_kernel (clusters of two CTAs, 256 x 256
 * tiles, tcgen05.mma cta_group::2), used from m_e = 1024; both draw their
 * (problem, product, tile) work items dynamically from a counter, so the
 * items in flight stay contiguous. A single call packs, multiplies and
 * updates C per product group; when the workspace holds all products it runs
 * them as two groups, the second group's packs and the first group's C
 * updates on pool streams beside the other group's GEMM, and a group's GEMM
 * as launches of about 24 rounds of items. The host-buffer call overlaps the
 * copies with the work (A in row halves and B in column chunks chased by
 * their packs, the GEMM in up to 2 x 2 blocks of tiles that start on half of
 * each operand, each block's C read back in column chunks behind its C
 * updates). Batched calls run waves of up
 * to 80 problems, one GEMM launch per tile kind per wave, waves alternating
 * between two workspace halves so a wave's packs overlap the previous wave.
 * Every path gives the same bits for a problem.
 */
#include "fmm_internal.h"
#include "sm103_ptx.cuh"

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <chrono>
#include <atomic>
#include <cstring>
#include <deque>
#include <mutex>
#include <utility>
#include <vector>

namespace {

constexpr int kTileM = 128;
constexpr int kTileN = 256;             /* N = 256: 128 clocks per MMA hide the accumulator dependency */
constexpr int kBK = 64;                 /* BF16 k elements per stage (128 bytes; 128 FP8 elements) */
constexpr int kStages = 4;
constexpr int kChunkKB = 16;            /* k-blocks per exact FP32 chunk: 1024 terms, |sum| <= 2^24 */
constexpr int kEpiWarps = 16;          /* four per TMEM lane quarter */
constexpr int kEpiCols = kTileN / 4;    /* columns per epilogue thread */
constexpr int kGemmThreads = 64 + 32 * kEpiWarps;  /* TMA warp, MMA warp, epilogue warps */
constexpr uint32_t kATileBytes = kTileM * kBK * 2;  /* 16 KB */
constexpr uint32_t kBTileBytes = kTileN * kBK * 2;  /* 32 KB */
constexpr uint32_t kStageBytes = kATileBytes + kBTileBytes;
constexpr int kTmemCols = 512;          /* 2 x 256 accumulator columns */
constexpr int kMaxKe = 16384;
constexpr int kRasterGroup = 12;        /* tile rows per raster band */
constexpr size_t kGemmSmem = (size_t)kStages * kStageBytes + 1024 + 256;

__host__ __device__ __forceinline__ int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

/* ------------------------------------------------------------ digits ---- */

/* E with 2^(E-1) <= b < 2^E for finite b > 0; 0 for b == 0. */
__device__ __forceinline__ int exp_above(double b)
{
    const uint64_t bits = (uint64_t)__double_as_longlong(b) & 0x7fffffffffffffffull;
    if (bits == 0) return 0;
    const int bexp = (int)(bits >> 52);
    if (bexp > 0) return bexp - 1022;
    return -1010 - __clzll((long long)bits);
}

/* Balanced base-2^DB digits of x relative to 2^E (|x| < 2^E): X =
 * round(x * 2^(DB*s-E-1)) (ties away from zero), |X| <= 2^(DB*s-1), split as
 * d[s-1], ..., d[1] in [-2^(DB-1), 2^(DB-1)) from the bottom and d[0] in
 * [-2^(DB-1), 2^(DB-1)]. DB = 8 (BF16 slices): every digit has at most 8
 * significant bits; DB = 5 (FP8-E4M3 slices): every digit is an integer of
 * magnitude at most 16, at most 4 significant bits. Both are exact.
 * The same digits in one step: Y = X + sum_{j < S-1} 2^(DB-1) * 2^(DB*j).
 * Adding 2^(DB-1) at every lower digit position turns the balanced digits
 * into plain DB-bit fields, so the low S-1 fields of Y are d[S-1] + 2^(DB-1),
 * ..., d[1] + 2^(DB-1) and floor(Y / 2^(DB(S-1))) is d[0]: the balanced
 * digits above, without a digit loop. Y is kept modulo 2^64 (its low fields
 * are exact); d[0] is (X >> DB(S-1)) plus the carry out of the low fields,
 * which stays exact for the 64-bit X of the largest S. */
struct Digits {
    int64_t X;
    uint64_t Y;
};

template <int S, int DB>
__host__ __device__ constexpr uint64_t digit_offset()
{
    uint64_t off = 0;
    for (int j = 0; j < S - 1; ++j) off |= (uint64_t)1 << (DB * j + DB - 1);
    return off;
}

template <int S, int DB>
__device__ __forceinline__ Digits split_offset(double x, int E)
{
    const uint64_t bits = (uint64_t)__double_as_longlong(x);
    const bool neg = (bits >> 63) != 0;
    const int bexp = (int)((bits >> 52) & 0x7ff);
    uint64_t mant = bits & 0x000fffffffffffffull;
    int ex;
    if (bexp == 0) ex = -1074; else { mant |= 0x0010000000000000ull; ex = bexp - 1075; }
    const int sh = ex + DB * S - E - 1;
    int64_t X;
    if (mant == 0 || sh < -62) X = 0;
    else if (sh >= 0) X = (int64_t)(mant << sh);
    else X = (int64_t)((mant + (1ull << (-sh - 1))) >> (-sh));
    if (neg) X = -X;
    return Digits{X, (uint64_t)X + digit_offset<S, DB>()};
}

/* digit t (0 = most significant) as an exact float. A lower digit is field
 * S-1-t of Y minus 2^(DB-1): the field is placed in the mantissa of 2^23 (one
 * byte permute for DB = 8, a shift and mask for DB = 5) and 2^23 + 2^(DB-1)
 * is subtracted, both exact. The top digit goes through the same 2^23-offset
 * conversion from its integer value. With t a compile-time constant after
 * unrolling, the field choice folds away. */
template <int S, int DB>
__device__ __forceinline__ float digit_f(const Digits& g, int t)
{
    constexpr int sh = DB * (S - 1);
    constexpr uint64_t kOff = digit_offset<S, DB>();
    constexpr uint64_t kMask = (1ull << sh) - 1;
    if (t == 0) {
        const int d = (int)(g.X >> sh) + (int)((((uint64_t)g.X & kMask) + kOff) >> sh);
        return __int_as_float(0x4B400000 + d) - 12582912.0f;   /* exact for |d| < 2^22 */
    }
    const int fi = S - 1 - t;
    if (DB == 8) {
        const uint32_t w = fi < 4 ? (uint32_t)g.Y : (uint32_t)(g.Y >> 32);
        return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u + (unsigned)(fi & 3))) - 8388736.0f;
    }
    const uint32_t field = (uint32_t)(g.Y >> (DB * fi)) & ((1u << DB) - 1);
    return __uint_as_float(0x4B000000u | field) - (8388608.0f + (float)(1 << (DB - 1)));
}

/* two floats that are exact in FP8-E4M3 (integers of magnitude <= 16) as a
 * packed e4m3x2 half-word, first value in the low byte */
__device__ __forceinline__ uint32_t pack_e4m3x2_exact(float lo, float hi)
{
    unsigned short h;
    asm("cvt.rn.satfinite.e4m3x2.f32 %0, %1, %2;" : "=h"(h) : "f"(hi), "f"(lo));
    return (uint32_t)h;
}

/* two floats that are exact in BF16 (at most 8 significant bits) as a packed
 * bf16x2 word, first value in the low half: their upper 16 bits */
__device__ __forceinline__ uint32_t pack_bf16x2_exact(float lo, float hi)
{
    return __byte_perm(__float_as_uint(lo), __float_as_uint(hi), 0x7632u);
}

/* Writes the S digit slices of 8 consecutive k elements: slice tt of the
 * element at (slice-0) element offset off lands at off + tt * slice_stride
 * of a BF16 (DB = 8, 16 bytes per slice) or FP8-E4M3 (DB = 5, 8 bytes per
 * slice) array. */
template <int S, int DB>
__device__ __forceinline__ void store_digits8(uint8_t* __restrict__ base, int64_t off, int64_t slice_stride,
                                              const Digits (&Y)[8])
{
#pragma unroll
    for (int tt = 0; tt < S; ++tt) {
        const int64_t e = off + (int64_t)tt * slice_stride;
        if (DB == 8) {
            uint32_t w[4];
#pragma unroll
            for (int h = 0; h < 4; ++h)
                w[h] = pack_bf16x2_exact(digit_f<S, DB>(Y[2 * h], tt), digit_f<S, DB>(Y[2 * h + 1], tt));
            *(uint4*)(base + 2 * e) = make_uint4(w[0], w[1], w[2], w[3]);
        } else {
            uint32_t h[4];
#pragma unroll
            for (int x = 0; x < 4; ++x)
                h[x] = pack_e4m3x2_exact(digit_f<S, DB>(Y[2 * x], tt), digit_f<S, DB>(Y[2 * x + 1], tt));
            *(uint2*)(base + e) = make_uint2(h[0] | (h[1] << 16), h[2] | (h[3] << 16));
        }
    }
}

/* v * 2^e, in at most two exact power-of-two multiplications. */
__device__ __forceinline__ double scale2(double v, int e)
{
    if (e > 1000) {
        v *= __longlong_as_double((long long)(1000 + 1023) << 52);
        e -= 1000;
    } else if (e < -1000) {
        v *= __longlong_as_double((long long)(-1000 + 1023) << 52);
        e += 1000;
    }
    return v * __longlong_as_double((long long)(e + 1023) << 52);
}

/* ------------------------------------------------- table access -------- */

struct Tab {
    int mt, kt, nt, R;
    const int* u_off; const int* v_off; const int* w_off;
    const int* u_ent; const int* v_ent; const int* w_ent;
    const int* wp_off; const int* wp_ent;
};

__host__ __device__ __forceinline__ Tab tab_view(const int* tab)
{
    Tab t;
    t.mt = tab[0]; t.kt = tab[1]; t.nt = tab[2]; t.R = tab[3];
    t.u_off = tab + FMM_ALG_HDR;
    t.v_off = t.u_off + (t.R + 1);
    t.w_off = t.v_off + (t.R + 1);
    t.u_ent = t.w_off + (t.R + 1);
    t.v_ent = t.u_ent + 2 * t.u_off[t.R];
    t.w_ent = t.v_ent + 2 * t.v_off[t.R];
    t.wp_off = t.w_ent + 2 * t.w_off[t.R];
    t.wp_ent = t.wp_off + (t.mt * t.nt + 1);
    return t;
}

/* ----------------------------------------------------- max kernels ----- */

/* amax[b*m + i] = max over the columns of k-block b of |A[i, :]| (as the bit
 * pattern of a non-negative double, which orders like the value). */
__device__ __forceinline__ void amax_body(const double* __restrict__ A, int64_t lda, int64_t m, int64_t k, int kt,
                                          unsigned long long* __restrict__ amax, int cols_per_block, int64_t bx,
                                          int by, int64_t bz, int64_t i_first = 0, int64_t i_end = -1)
{
    const int64_t i = i_first + bx * (int64_t)blockDim.x + threadIdx.x;
    const int b = by;
    if (i >= (i_end < 0 ? m : i_end)) return;
    int64_t co, cl;
    fmm_part_geom(k, kt, b, &co, &cl);
    const int64_t c0 = bz * cols_per_block;
    if (c0 >= cl) return;
    const int64_t c1 = cl < c0 + cols_per_block ? cl : c0 + cols_per_block;
    const double* col = A + i + (co + c0) * lda;
    const int nc = (int)(c1 - c0);
    unsigned long long mx = 0;
    int c = 0;
    for (; c + 8 <= nc; c += 8) {   /* eight independent loads in flight */
        unsigned long long v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u)
            v[u] = (unsigned long long)__double_as_longlong(__ldg(col + (int64_t)(c + u) * lda)) &
                   0x7fffffffffffffffull;
#pragma unroll
        for (int u = 0; u < 8; ++u) mx = v[u] > mx ? v[u] : mx;
    }
    for (; c < nc; ++c) {
        const unsigned long long v =
            (unsigned long long)__double_as_longlong(__ldg(col + (int64_t)c * lda)) & 0x7fffffffffffffffull;
        mx = v > mx ? v : mx;
    }
    atomicMax(&amax[(int64_t)b * m + i], mx);
}

/* the rows [i_first, i_end) of A */
__global__ void amax_kernel(const double* __restrict__ A, int64_t lda, int64_t m, int64_t k,
                            int kt, unsigned long long* __restrict__ amax, int cols_per_block, int64_t i_first,
                            int64_t i_end)
{
    amax_body(A, lda, m, k, kt, amax, cols_per_block, blockIdx.x, blockIdx.y, blockIdx.z, i_first, i_end);
}

/* bmax[b*n + j] = max over the rows of k-block b of |B[:, j]| for the columns
 * j in [c0, c1); one warp per (j, b). */
__device__ __forceinline__ void bmax_body(const double* __restrict__ B, int64_t ldb, int64_t k, int64_t n, int kt,
                                          unsigned long long* __restrict__ bmax, int64_t c0, int64_t c1, int64_t bx)
{
    const int64_t w = (bx * (int64_t)blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x % 32;
    const int64_t nc = c1 - c0;
    if (w >= nc * kt) return;
    const int64_t j = c0 + w % nc;
    const int b = (int)(w / nc);
    int64_t ro, rl;
    fmm_part_geom(k, kt, b, &ro, &rl);
    unsigned long long mx = 0;
    for (int64_t p = lane; p < rl; p += 32) {
        const unsigned long long v =
            (unsigned long long)__double_as_longlong(B[ro + p + j * ldb]) & 0x7fffffffffffffffull;
        mx = v > mx ? v : mx;
    }
#pragma unroll
    for (int o = 16; o > 0; o /= 2) {
        const unsigned long long y = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = y > mx ? y : mx;
    }
    if (lane == 0) bmax[(int64_t)b * n + j] = mx;
}

__global__ void bmax_kernel(const double* __restrict__ B, int64_t ldb, int64_t k, int64_t n,
                            int kt, unsigned long long* __restrict__ bmax, int64_t c0, int64_t c1)
{
    bmax_body(B, ldb, k, n, kt, bmax, c0, c1, blockIdx.x);
}

/* Row exponents of S_r (index < m_pad) and column exponents of T_r (index
 * m_pad + j) for the products r = r0 + blockIdx.y of a group, into
 * e_row[q][m_pad] and f_col[q][n_pad]; a launch covers the indices
 * [first, end), so the row side (needs only amax) and the column side (needs
 * only bmax) can run on different streams. */
__device__ __forceinline__ void exps_body(const int* __restrict__ tab, int r0, int64_t m, int64_t n, int64_t k,
                                          int64_t m_pad, int64_t n_pad, const unsigned long long* __restrict__ amax,
                                          const unsigned long long* __restrict__ bmax, int* __restrict__ e_row,
                                          int* __restrict__ f_col, int64_t first, int64_t end, int64_t bx, int by)
{
    const Tab t = tab_view(tab);
    const int r = r0 + by;
    e_row += (int64_t)by * m_pad;
    f_col += (int64_t)by * n_pad;
    const int64_t me = (m + t.mt - 1) / t.mt, ne = (n + t.nt - 1) / t.nt;
    const int64_t idx = first + bx * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= end) return;
    if (idx < m_pad) {
        const int64_t i = idx;
        double bnd = 0.0;
        bool first = true;
        if (i < me) {
            for (int e = t.u_off[r]; e < t.u_off[r + 1]; ++e) {
                const int part = t.u_ent[2 * e];
                const double c = fabs((double)t.u_ent[2 * e + 1]);
                int64_t ro, rl;
                fmm_part_geom(m, t.mt, part / t.kt, &ro, &rl);
                if (i >= rl) continue;
                const double mx = __longlong_as_double((long long)amax[(int64_t)(part % t.kt) * m + ro + i]);
                bnd = first ? c * mx : fma(c, mx, bnd);
                first = false;
            }
        }
        e_row[i] = exp_above(bnd);
    } else if (idx < m_pad + n_pad) {
        const int64_t j = idx - m_pad;
        double bnd = 0.0;
        bool first = true;
        if (j < ne) {
            for (int e = t.v_off[r]; e < t.v_off[r + 1]; ++e) {
                const int part = t.v_ent[2 * e];
                const double c = fabs((double)t.v_ent[2 * e + 1]);
                int64_t co, cl;
                fmm_part_geom(n, t.nt, part % t.nt, &co, &cl);
                if (j >= cl) continue;
                const double mx = __longlong_as_double((long long)bmax[(int64_t)(part / t.nt) * n + co + j]);
                bnd = first ? c * mx : fma(c, mx, bnd);
                first = false;
            }
        }
        f_col[j] = exp_above(bnd);
    }
    (void)k;
}

__global__ void exps_kernel(const int* __restrict__ tab, int r0, int64_t m, int64_t n, int64_t k,
                            int64_t m_pad, int64_t n_pad,
                            const unsigned long long* __restrict__ amax,
                            const unsigned long long* __restrict__ bmax,
                            int* __restrict__ e_row, int* __restrict__ f_col, int64_t first, int64_t end)
{
    exps_body(tab, r0, m, n, k, m_pad, n_pad, amax, bmax, e_row, f_col, first, end, blockIdx.x, blockIdx.y);
}

/* ----------------------------------------------------- pack kernels ---- */

constexpr int kPackMaxEnt = 256;

/* one sub-block term of a packing sum: base pointer, extent, coefficient as
 * a double and its kind (0: +1, 1: -1, 2: other), so the per-element code
 * does no conversion and no FP64 compare */
struct PEnt {
    const double* base;
    double coef;
    int rows, cols;
    int kind;
    int pad;
};

__device__ __forceinline__ PEnt make_pent(const double* base, int64_t rows, int64_t cols, int c)
{
    PEnt x;
    x.base = base;
    x.coef = (double)c;
    x.rows = (int)rows;
    x.cols = (int)cols;
    x.kind = c == 1 ? 0 : (c == -1 ? 1 : 2);
    x.pad = 0;
    return x;
}

/* first term of a packing sum over a thread's values: s[t] = c * s[t],
 * exact like the FP64 product; sign flips for c = +-1 keep it off the FP64
 * pipe, and the branch (uniform over the CTA) is taken once for all values */
template <int N>
__device__ __forceinline__ void scale_first(const PEnt& x, double (&s)[N])
{
    if (x.kind == 1) {
#pragma unroll
        for (int t = 0; t < N; ++t)
            s[t] = __longlong_as_double(__double_as_longlong(s[t]) ^ (long long)0x8000000000000000ull);
    } else if (x.kind == 2) {
#pragma unroll
        for (int t = 0; t < N; ++t) s[t] = x.coef * s[t];
    }
}

/* A side, all products r0 .. r0+np-1 of a group in one launch: CTA (q, tile)
 * forms the tile of ROWS rows x 64 k of S_r, r = r0 + q, and writes its digits
 * row-major (K-major) into slices sa[q][t][m_pad][k_pad]. The product index
 * runs fastest in the block order, so the products at one tile position run
 * together and read their shared A sub-block tiles through L2 once. ROWS = 64
 * (256 threads) for single calls; ROWS = 32 (128 threads, 25 KB of shared
 * memory, at most 64 registers) for batched waves, small enough to run on an
 * SM beside a resident GEMM CTA. */
template <int S, int DB, int ROWS>
__device__ __forceinline__ void pack_a_body(const int* __restrict__ tab, int r0, int np, const double* __restrict__ A,
                                            int64_t lda, int64_t m, int64_t k, int64_t m_pad, int64_t k_pad,
                                            const int* __restrict__ e_row, uint8_t* __restrict__ sa, int64_t bx,
                                            int64_t by, int64_t i_first = 0)
{
    __shared__ double Sf[64][ROWS + 1];
    __shared__ PEnt ent[kPackMaxEnt];
    const Tab t = tab_view(tab);
    const int64_t me = (m + t.mt - 1) / t.mt, ke = (k + t.kt - 1) / t.kt;
    const int q = (int)(bx % np);
    const int r = r0 + q;
    const int64_t i0 = i_first + (bx / np) * ROWS, p0 = by * 64;
    e_row += (int64_t)q * m_pad;
    const int64_t slice0 = (int64_t)q * S * m_pad * k_pad;   /* element offset of this product */
    const int eb = t.u_off[r], ne_ = t.u_off[r + 1] - eb;
    for (int e = threadIdx.x; e < ne_; e += blockDim.x) {
        const int part = t.u_ent[2 * (eb + e)];
        int64_t ro, rl, co, cl;
        fmm_part_geom(m, t.mt, part / t.kt, &ro, &rl);
        fmm_part_geom(k, t.kt, part % t.kt, &co, &cl);
        ent[e] = make_pent(A + ro + co * lda, rl, cl, t.u_ent[2 * (eb + e) + 1]);
    }
    __syncthreads();
    /* 16 elements per thread in two halves of 8: each term's 8 loads go out
     * together, and the first term's coefficient (uniform over the CTA) is
     * applied once after them */
    const int li = threadIdx.x % ROWS, kq = threadIdx.x / ROWS;   /* row, k offset 0..3 */
    const int64_t gi = i0 + li;
    const bool row_ok = ne_ > 0 && gi < me;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        double v8[8];
#pragma unroll
        for (int y = 0; y < 8; ++y) v8[y] = 0.0;
        if (row_ok) {
            /* term e + 1's loads go out before term e's FMAs; per term, one
             * row test and one k limit, then a pointer step of 4 columns per
             * element (no per-element index arithmetic) */
            const int64_t st4 = 4 * lda;
            auto load8 = [&](const PEnt& x, double (&d)[8]) {
                const bool rok = gi < x.rows;
                const int64_t kl = (ke < x.cols ? ke : x.cols) - (p0 + kq + 32 * h);   /* valid while 4y < kl */
                const double* pt = x.base + gi + (p0 + kq + 32 * h) * lda;
#pragma unroll
                for (int y = 0; y < 8; ++y) {
                    d[y] = (rok && 4 * y < kl) ? __ldg(pt) : 0.0;
                    pt += st4;
                }
            };
            double nx[8];
            load8(ent[0], v8);
            if (ne_ > 1) load8(ent[1], nx);
            scale_first(ent[0], v8);
            for (int e = 1; e < ne_; ++e) {
                double cur[8];
#pragma unroll
                for (int y = 0; y < 8; ++y) cur[y] = nx[y];
                if (e + 1 < ne_) load8(ent[e + 1], nx);
                const double c = ent[e].coef;
#pragma unroll
                for (int y = 0; y < 8; ++y) v8[y] = fma(c, cur[y], v8[y]);
            }
        }
#pragma unroll
        for (int y = 0; y < 8; ++y) Sf[kq + 4 * (8 * h + y)][li] = v8[y];
    }
    __syncthreads();
    /* thread -> (row, 8 consecutive k): 4 rows x 128 bytes per warp store */
    const int kg = threadIdx.x % 8;
    for (int rr = threadIdx.x / 8; rr < ROWS; rr += ROWS / 2) {
        const int64_t gi = i0 + rr;
        const int E = e_row[gi];
        Digits Y[8];
#pragma unroll
        for (int x = 0; x < 8; ++x) Y[x] = split_offset<S, DB>(Sf[kg * 8 + x][rr], E);
        store_digits8<S, DB>(sa, slice0 + gi * k_pad + p0 + kg * 8, m_pad * k_pad, Y);
    }
}

template <int S, int DB, int ROWS>
__global__ void __launch_bounds__(ROWS * 4, ROWS == 64 ? 4 : 8)
pack_a_kernel(const int* __restrict__ tab, int r0, int np, const double* __restrict__ A, int64_t lda,
              int64_t m, int64_t k, int64_t m_pad, int64_t k_pad,
              const int* __restrict__ e_row, uint8_t* __restrict__ sa, int64_t i_first)
{
    pack_a_body<S, DB, ROWS>(tab, r0, np, A, lda, m, k, m_pad, k_pad, e_row, sa, blockIdx.x, blockIdx.y, i_first);
}

/* B side, all products of a group: CTA (q, tile) forms the tile of COLS
 * columns x 64 k of T_r, r = r0 + q (column j of T_r is contiguous in k
 * already), and writes its digits into slices sb[q][t][n_pad][k_pad];
 * product index fastest, as on the A side. COLS = 32 (256 threads) for single
 * calls, 16 (128 threads, at most 64 registers) for batched waves. */
template <int S, int DB, int COLS>
__device__ __forceinline__ void pack_b_body(const int* __restrict__ tab, int r0, int np, const double* __restrict__ B,
                                            int64_t ldb, int64_t k, int64_t n, int64_t n_pad, int64_t k_pad,
                                            const int* __restrict__ f_col, uint8_t* __restrict__ sb, int64_t j_first,
                                            int64_t bx, int64_t by)
{
    __shared__ PEnt ent[kPackMaxEnt];
    const Tab t = tab_view(tab);
    const int64_t ne = (n + t.nt - 1) / t.nt, ke = (k + t.kt - 1) / t.kt;
    const int q = (int)(bx % np);
    const int r = r0 + q;
    f_col += (int64_t)q * n_pad;
    const int64_t slice0 = (int64_t)q * S * n_pad * k_pad;
    const int eb = t.v_off[r], ne_ = t.v_off[r + 1] - eb;
    for (int e = threadIdx.x; e < ne_; e += blockDim.x) {
        const int part = t.v_ent[2 * (eb + e)];
        int64_t ro, rl, co, cl;
        fmm_part_geom(k, t.kt, part / t.nt, &ro, &rl);
        fmm_part_geom(n, t.nt, part % t.nt, &co, &cl);
        ent[e] = make_pent(B + ro + co * ldb, rl, cl, t.v_ent[2 * (eb + e) + 1]);
    }
    __syncthreads();
    const int kg = threadIdx.x % 8;
    const int64_t gj = j_first + (bx / np) * COLS + threadIdx.x / 8;
    const int64_t p0 = by * 64 + kg * 8;
    double v8[8];
#pragma unroll
    for (int x = 0; x < 8; ++x) v8[x] = 0.0;
    if (ne_ > 0 && gj < ne) {
        /* term e + 1's loads go out before term e's FMAs; per term, one
         * column test and one k limit, then 8 contiguous values at fixed
         * offsets from one pointer */
        auto load8 = [&](const PEnt& x, double (&d)[8]) {
            const int64_t kl = (ke < x.rows ? ke : x.rows) - p0;   /* valid while y < kl */
            const bool cok = gj < x.cols;
            const double* pt = x.base + gj * ldb + p0;
#pragma unroll
            for (int y = 0; y < 8; ++y) d[y] = (cok && y < kl) ? __ldg(pt + y) : 0.0;
        };
        double nx[8];
        load8(ent[0], v8);
        if (ne_ > 1) load8(ent[1], nx);
        scale_first(ent[0], v8);
        for (int e = 1; e < ne_; ++e) {
            double cur[8];
#pragma unroll
            for (int y = 0; y < 8; ++y) cur[y] = nx[y];
            if (e + 1 < ne_) load8(ent[e + 1], nx);
            const double c = ent[e].coef;
#pragma unroll
            for (int y = 0; y < 8; ++y) v8[y] = fma(c, cur[y], v8[y]);
        }
    }
    const int F = f_col[gj];
    Digits Y[8];
#pragma unroll
    for (int x = 0; x < 8; ++x) Y[x] = split_offset<S, DB>(v8[x], F);
    store_digits8<S, DB>(sb, slice0 + gj * k_pad + p0, n_pad * k_pad, Y);
}

template <int S, int DB, int COLS>
__global__ void __launch_bounds__(COLS * 8, COLS == 32 ? 4 : 8)
pack_b_kernel(const int* __restrict__ tab, int r0, int np, const double* __restrict__ B, int64_t ldb,
              int64_t k, int64_t n, int64_t n_pad, int64_t k_pad,
              const int* __restrict__ f_col, uint8_t* __restrict__ sb, int64_t j_first)
{
    pack_b_body<S, DB, COLS>(tab, r0, np, B, ldb, k, n, n_pad, k_pad, f_col, sb, j_first, blockIdx.x, blockIdx.y);
}

/* Which packs a launch_packs call issues: both sides, or one side only; the
 * A side over the S_r rows [ia0, ia1) (multiples of 64, or ia1 = m_pad), the
 * B side over the T_r columns [jb0, jb1) (multiples of 32, or jb1 = n_pad). */
struct PackSel {
    bool a = true, b = true;
    int64_t ia0 = 0, ia1 = -1;
    int64_t jb0 = 0, jb1 = -1;
    bool small = false;   /* the 128-thread tiles that fit beside a resident GEMM CTA */
};

template <int S, int DB>
void launch_packs_t(const int* tab, int r, int np, const double* A, int64_t lda, const double* B, int64_t ldb,
                    int64_t m, int64_t n, int64_t k, int64_t m_pad, int64_t n_pad, int64_t k_pad,
                    const int* e_row, const int* f_col, uint8_t* sa, uint8_t* sb, cudaStream_t st,
                    cudaStream_t st_b, const PackSel& sel)
{
    const int64_t i1 = sel.ia1 < 0 ? m_pad : sel.ia1;
    const int rows = sel.small ? 32 : 64;
    const dim3 ka((unsigned)(np * ((i1 - sel.ia0 + rows - 1) / rows)), (unsigned)(k_pad / 64));
    if (sel.a && i1 > sel.ia0 && sel.small)
        pack_a_kernel<S, DB, 32><<<ka, 128, 0, st>>>(tab, r, np, A, lda, m, k, m_pad, k_pad, e_row, sa, sel.ia0);
    else if (sel.a && i1 > sel.ia0)
        pack_a_kernel<S, DB, 64><<<ka, 256, 0, st>>>(tab, r, np, A, lda, m, k, m_pad, k_pad, e_row, sa, sel.ia0);
    const int64_t j1 = sel.jb1 < 0 ? n_pad : sel.jb1;
    if (!sel.b || j1 <= sel.jb0) return;
    const int cols = sel.small ? 16 : 32;
    const dim3 kb((unsigned)(np * ((j1 - sel.jb0 + cols - 1) / cols)), (unsigned)(k_pad / 64));
    if (sel.small)
        pack_b_kernel<S, DB, 16><<<kb, 128, 0, st_b>>>(tab, r, np, B, ldb, k, n, n_pad, k_pad, f_col, sb, sel.jb0);
    else
        pack_b_kernel<S, DB, 32><<<kb, 256, 0, st_b>>>(tab, r, np, B, ldb, k, n, n_pad, k_pad, f_col, sb, sel.jb0);
}

/* digit slices of the products r .. r+np-1 (exponents already in place);
 * fmt 0: BF16 (s = 2..8), fmt 1: FP8-E4M3 (s = 2..12); the B side on st_b */
void launch_packs(int fmt, int s, const int* tab, int r, int np, const double* A, int64_t lda, const double* B,
                  int64_t ldb, int64_t m, int64_t n, int64_t k, int64_t m_pad, int64_t n_pad,
                  int64_t k_pad, const int* e_row, const int* f_col, uint8_t* sa, uint8_t* sb,
                  cudaStream_t st, cudaStream_t st_b, const PackSel& sel = PackSel())
{
#define FMM_PACKS(S_, DB_) \
    launch_packs_t<S_, DB_>(tab, r, np, A, lda, B, ldb, m, n, k, m_pad, n_pad, k_pad, e_row, f_col, sa, sb, st, \
                            st_b, sel)
    if (fmt == 0) {
        switch (s) {
        case 2: FMM_PACKS(2, 8); break;
        case 3: FMM_PACKS(3, 8); break;
        case 4: FMM_PACKS(4, 8); break;
        case 5: FMM_PACKS(5, 8); break;
        case 6: FMM_PACKS(6, 8); break;
        case 7: FMM_PACKS(7, 8); break;
        default: FMM_PACKS(8, 8); break;
        }
    } else {
        switch (s) {
        case 2: FMM_PACKS(2, 5); break;
        case 3: FMM_PACKS(3, 5); break;
        case 4: FMM_PACKS(4, 5); break;
        case 5: FMM_PACKS(5, 5); break;
        case 6: FMM_PACKS(6, 5); break;
        case 7: FMM_PACKS(7, 5); break;
        case 8: FMM_PACKS(8, 5); break;
        case 9: FMM_PACKS(9, 5); break;
        case 10: FMM_PACKS(10, 5); break;
        case 11: FMM_PACKS(11, 5); break;
        default: FMM_PACKS(12, 5); break;
        }
    }
#undef FMM_PACKS
}

/* ------------------------------------------------------ GEMM kernel ---- */

/* (double)z * 2^e for |z| < 2^62 in integer arithmetic (round to nearest
 * even, then exponent offset), identical to the FP64 conversion and
 * power-of-two scaling whenever the result is a normal number; other cases
 * take the FP64 route. Keeps the per-element FP64 work to the C updates. */
/* the FP64 route for results outside the normal range, kept out of line so
 * the common path carries no FP64 instruction */
__device__ __noinline__ double i64_to_double_scaled_slow(int64_t z, int e)
{
    return scale2((double)z, e);
}

__device__ __forceinline__ double i64_to_double_scaled(int64_t z, int e)
{
    if (z == 0) return 0.0;
    const uint64_t sign = z < 0 ? 0x8000000000000000ull : 0ull;
    uint64_t u = z < 0 ? (uint64_t)(-z) : (uint64_t)z;
    int p = 63 - __clzll((long long)u);
    uint64_t m;
    if (p <= 52) {
        m = u << (52 - p);
    } else {
        const int sh = p - 52;
        m = u >> sh;
        const uint64_t rem = u & ((1ull << sh) - 1), half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (m & 1))) {
            ++m;
            if (m == (1ull << 53)) { m >>= 1; ++p; }
        }
    }
    const int be = p + 1023 + e;
    if (be < 1 || be > 2046) return i64_to_double_scaled_slow(z, e);
    return __longlong_as_double((long long)(sign | ((uint64_t)be << 52) | (m & 0x000fffffffffffffull)));
}

/* One problem of a GEMM launch: the digit slices of a product group of one
 * FMM GEMM and where its level accumulators go. */
struct GemmProblem {
    CUtensorMap tmA;      /* A slices [product][s][m_pad][k_pad], box 64 x 128 */
    CUtensorMap tmB;      /* B slices [product][s][n_pad][k_pad], box 64 x 256 */
    int64_t* Z;           /* [product][n_pad][m_pad] int64 level accumulators */
    int s;                /* slices */
    int zlevel;           /* G: the level whose unit Z counts in */
    int nkb;              /* k_pad / kbe */
    int kbe;              /* k elements per 128-byte stage row: 64 (BF16) or 128 (FP8) */
    int db;               /* digit bits: 8 (BF16) or 5 (FP8-E4M3) */
    int fmt;              /* 0: BF16 slices, kind::f16; 1: FP8-E4M3 slices, kind::f8f6f4 */
    int m_pad, n_pad;     /* rows per slice in the A / B slice arrays */
    int tiles_m, tiles_n; /* per product */
    int item_begin;       /* first work item of this problem in the launch */
};

/* problems per GEMM launch: the table travels as a kernel parameter, whose
 * space is 32764 bytes (a GemmProblem is 384 bytes with its two 128-byte
 * aligned tensor maps) */
constexpr int kMaxLaunchProblems = 80;

/* Everything a launch needs, passed by value (tensor maps included), so a
 * launch copies nothing to the device and can be captured in a graph. */
struct GemmLaunch {
    int nprob;
    int nitems;           /* sum over problems of products * tiles */
    int* err;
    unsigned int* sched;  /* pair kernel: next work item, zero at launch */
    GemmProblem prob[kMaxLaunchProblems];
};
static_assert(sizeof(GemmLaunch) <= 32764, "GemmLaunch must fit the kernel parameter space");

__device__ __forceinline__ int level_pairs(int g, int s) { return min(s, g - 1) - max(1, g - s) + 1; }

/* Work item b -> problem, product and tile: problems in order, products in
 * order within a problem, then a grouped raster of kRasterGroup tile rows so
 * the CTAs resident together share slice panels in L2. */
struct Item {
    int p, r, tile_m, tile_n;
};

__device__ __forceinline__ Item decode_item(const GemmLaunch& L, int b, int raster = kRasterGroup)
{
    int p = 0, hi = L.nprob - 1;        /* last problem with item_begin <= b */
    while (p < hi) {
        const int mid = (p + hi + 1) / 2;
        if (L.prob[mid].item_begin <= b) p = mid; else hi = mid - 1;
    }
    const GemmProblem& P = L.prob[p];
    const int local = b - P.item_begin;
    const int per_prod = P.tiles_m * P.tiles_n;
    Item it;
    it.p = p;
    it.r = local / per_prod;
    const int id = local % per_prod;
    const int per_group = raster * P.tiles_n;
    const int grp = id / per_group, first_m = grp * raster;
    const int gm = min(P.tiles_m - first_m, raster);
    const int in_grp = id % per_group;
    it.tile_m = first_m + in_grp % gm;
    it.tile_n = in_grp / gm;
    return it;
}

constexpr int kSchedSlots = 4;
/* readers of each ring slot: the even CTA's MMA thread, every epilogue warp of
 * both CTAs, the odd CTA's producer */
constexpr int kSchedConsumers = 1 + 2 * kEpiWarps + 1;

/* Consumer side of the pair kernel's work-item ring: the even CTA's producer
 * takes items from a global counter and writes each into slot `slot` of both
 * CTAs' rings; a consumer waits for the slot, reads it and reports it read on
 * the even CTA's sempty barrier (release at cluster scope: the read is done
 * before the slot can be written again). */
struct ItemRing {
    uint32_t base;   /* shared-memory address of sfull[0]; sempty and sitem follow */
    int slot;
    uint32_t ph;

    __device__ __forceinline__ uint32_t full_at() const { return base + 8u * (uint32_t)slot; }
    __device__ __forceinline__ uint32_t empty_at() const { return base + 8u * (uint32_t)(kSchedSlots + slot); }
    __device__ __forceinline__ uint32_t item_at() const { return base + 16u * kSchedSlots + 4u * (uint32_t)slot; }
    __device__ __forceinline__ void next()
    {
        if (++slot == kSchedSlots) { slot = 0; ph ^= 1; }
    }
    __device__ __forceinline__ bool take(int* b, volatile int* abort_flag, int* err, int code)
    {
        if (!sm103::mbar_wait_acq_cluster_u32(full_at(), ph, abort_flag, err, code)) return false;
        *b = (int)sm103::ld_shared_u32(item_at());
        sm103::mbar_arrive_release_cluster(sm103::mapa(empty_at(), 0));
        next();
        return true;
    }
    /* lane 0 of a warp takes the slot and hands the item to the other lanes */
    __device__ __forceinline__ bool take_warp(int* b, int lane, volatile int* abort_flag, int* err, int code)
    {
        int got = 0, v = 0;
        if (lane == 0) {
            got = take(&v, abort_flag, err, code) ? 1 : 0;
        } else {
            next();
        }
        got = __shfl_sync(0xffffffffu, got, 0);
        *b = __shfl_sync(0xffffffffu, v, 0);
        return got != 0;
    }
};

/* Persistent GEMM over a list of work items (problem, product of its group,
 * 128 x 256 output tile), drawn dynamically: the producer takes the next item
 * from L.sched and passes it to the other roles through a CTA-local item
 * ring, so the CTAs' items in flight stay contiguous. One CTA per
 * SM: warp 0 issues the TMA loads of the digit-slice tiles, warp 1 the
 * tcgen05.mma (M=128, N=256, K=16 BF16 or K=32 FP8 per the item's problem:
 * 128 clocks per MMA hide the accumulator dependency), warps 2..17 drain
 * each exact chunk (16 stage rows: 1024 BF16 or 2048 FP8 terms) from the
 * double-buffered TMEM accumulator into int32 level sums and fold finished
 * levels into the product's 64-bit Z tile in global memory. The pipeline,
 * TMEM allocation and barrier phases run on across items, so one item's last
 * fold overlaps the next item's first MMAs. */
__global__ void __launch_bounds__(kGemmThreads, 1)
split_gemm_kernel(const __grid_constant__ GemmLaunch L)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* sA = smem;
    uint8_t* sB = smem + kStages * kATileBytes;
    uint64_t* full = (uint64_t*)(smem + kStages * kStageBytes);
    uint64_t* empty = full + kStages;
    uint64_t* accf = empty + kStages;
    uint64_t* acce = accf + 2;
    uint64_t* drain = acce + 2;
    uint64_t* sfull = drain + 1;                  /* item ring: slot written */
    uint64_t* sempty = sfull + kSchedSlots;       /* item ring: slot read by every consumer */
    int* sitem = (int*)(sempty + kSchedSlots);
    uint32_t* tmem_slot = (uint32_t*)(sitem + kSchedSlots);
    volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;

    if (threadIdx.x == 0) {
        for (int i = 0; i < kStages; ++i) { sm103::mbar_init(&full[i], 1); sm103::mbar_init(&empty[i], 1); }
        for (int i = 0; i < 2; ++i) { sm103::mbar_init(&accf[i], 1); sm103::mbar_init(&acce[i], kEpiWarps); }
        sm103::mbar_init(drain, 1);
        for (int i = 0; i < kSchedSlots; ++i) {
            sm103::mbar_init(&sfull[i], 1);
            sm103::mbar_init(&sempty[i], 1 + kEpiWarps);   /* the MMA thread and every epilogue warp */
        }
        *abort_flag = 0;
        sm103::fence_mbar_init();
    }
    if (warp == 1) { sm103::tmem_alloc(tmem_slot, kTmemCols); sm103::tmem_relinquish(); }
    sm103::tc_fence_before();
    __syncthreads();
    sm103::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        /* ---------------- TMA producer ---------------- */
        if (lane == 0) {
            int st = 0;
            uint32_t ph = 0;
            uint32_t armed = 0;  /* stages armed in the current pass (bit mask) */
            bool ok = true;
            int last_p = -1;
            ItemRing ring{sm103::smem_u32(sfull), 0, 0};
            for (;;) {
                /* the producer takes the next item from L.sched and publishes it */
                if (!sm103::mbar_wait_acq_cluster_u32(ring.empty_at(), ring.ph ^ 1, abort_flag, L.err, 7)) {
                    ok = false;
                    break;
                }
                int b = (int)atomicAdd(L.sched, 1u);
                if (b >= L.nitems) b = -1;
                sitem[ring.slot] = b;
                sm103::mbar_arrive(&sfull[ring.slot]);
                ring.next();
                if (b < 0) break;
                const Item it = decode_item(L, b);
                const GemmProblem& P = L.prob[it.p];
                if (it.p != last_p) { sm103::prefetch_tmap(&P.tmA); sm103::prefetch_tmap(&P.tmB); last_p = it.p; }
                const int s = P.s, nkb = P.nkb;
                const int arow = it.r * s * P.m_pad + it.tile_m * kTileM;
                const int brow = it.r * s * P.n_pad + it.tile_n * kTileN;
                /* Pair order: t ascending in even levels and descending in odd
                 * ones, so the last pair of a level and the first of the next
                 * share a slice ((1,2)->(1,3), (3,1)->(4,1), ...), and k runs
                 * forward and backward on alternate pairs, so a shared slice's
                 * most recently loaded blocks are read again first, while they
                 * are still in L2. The MMA side only counts stages; every
                 * chunk sum is exact in any order. (An L2 prefetch of the boxes
                 * eight stages ahead measured 3x slower, with 7x the DRAM
                 * reads.) */
                int pi = 0;
                for (int g = 2; g <= s + 1 && ok; ++g) {
                    const int tlo = max(1, g - s), thi = min(s, g - 1);
                    for (int x = 0; x <= thi - tlo && ok; ++x, ++pi) {
                        const int t = (g & 1) ? thi - x : tlo + x;
                        const int u = g - t;
                        for (int y = 0; y < nkb; ++y) {
                            const int kb = (pi & 1) ? nkb - 1 - y : y;
                            if (!sm103::mbar_wait(&empty[st], ph ^ 1, abort_flag, L.err, 1)) { ok = false; break; }
                            sm103::mbar_arrive_expect_tx(&full[st], kStageBytes);
                            sm103::tma_load_2d(sA + st * kATileBytes, &P.tmA, &full[st], kb * P.kbe,
                                               arow + (t - 1) * P.m_pad);
                            sm103::tma_load_2d(sB + st * kBTileBytes, &P.tmB, &full[st], kb * P.kbe,
                                               brow + (u - 1) * P.n_pad);
                            armed |= 1u << st;
                            if (++st == kStages) { st = 0; ph ^= 1; armed = 0; }
                        }
                    }
                }
            }
            if (!ok) {
                /* let every load already issued land before the CTA exits */
                for (int i = 0; i < kStages; ++i) {
                    const uint32_t par = (armed >> i) & 1u ? ph : ph ^ 1;
                    uint64_t t0 = sm103::globaltimer();
                    while (!sm103::mbar_try_wait(&full[i], par) &&
                           sm103::globaltimer() - t0 < sm103::kWaitLimitNs) {}
                }
            }
        }
    } else if (warp == 1) {
        /* ---------------- MMA issuer ---------------- */
        if (lane == 0) {
            constexpr uint32_t idesc16 = sm103::idesc_bf16_f32(kTileM, kTileN);
            constexpr uint32_t idesc8 = sm103::idesc_e4m3_f32(kTileM, kTileN);
            int st = 0, buf = 0;
            uint32_t ph = 0, aph = 0;
            bool ok = true;
            ItemRing ring{sm103::smem_u32(sfull), 0, 0};
            for (;;) {
                int b;
                if (!ring.take(&b, abort_flag, L.err, 8)) { ok = false; break; }
                if (b < 0) break;
                const Item it = decode_item(L, b);
                const int s = L.prob[it.p].s, nkb = L.prob[it.p].nkb, fmt = L.prob[it.p].fmt;
                for (int g = 2; g <= s + 1 && ok; ++g) {
                    const int level_kb = level_pairs(g, s) * nkb;
                    int jl = 0;
                    for (int t = max(1, g - s); t <= min(s, g - 1) && ok; ++t)
                        for (int kb = 0; kb < nkb; ++kb) {
                            if (jl % kChunkKB == 0) {
                                if (!sm103::mbar_wait(&acce[buf], aph ^ 1, abort_flag, L.err, 2)) { ok = false; break; }
                                sm103::tc_fence_after();
                            }
                            if (!sm103::mbar_wait(&full[st], ph, abort_flag, L.err, 3)) { ok = false; break; }
                            sm103::tc_fence_after();
                            const uint32_t a0 = sm103::smem_u32(sA + st * kATileBytes);
                            const uint32_t b0 = sm103::smem_u32(sB + st * kBTileBytes);
                            /* four MMAs per 128-byte stage row: K = 16 BF16 or 32 FP8
                             * elements each, 32 bytes apart */
                            if (fmt) {
#pragma unroll
                                for (int kk = 0; kk < 4; ++kk)
                                    sm103::mma_f8(tmem + buf * kTileN, sm103::smem_desc_sw128(a0 + kk * 32),
                                                  sm103::smem_desc_sw128(b0 + kk * 32), idesc8,
                                                  (jl % kChunkKB != 0 || kk != 0) ? 1u : 0u);
                            } else {
#pragma unroll
                                for (int kk = 0; kk < 4; ++kk)
                                    sm103::mma_bf16(tmem + buf * kTileN, sm103::smem_desc_sw128(a0 + kk * 32),
                                                    sm103::smem_desc_sw128(b0 + kk * 32), idesc16,
                                                    (jl % kChunkKB != 0 || kk != 0) ? 1u : 0u);
                            }
                            sm103::mma_commit(&empty[st]);
                            if (++st == kStages) { st = 0; ph ^= 1; }
                            ++jl;
                            if (jl % kChunkKB == 0 || jl == level_kb) {
                                sm103::mma_commit(&accf[buf]);
                                buf ^= 1;
                                if (buf == 0) aph ^= 1;
                            }
                        }
                }
            }
            /* all issued MMAs complete before TMEM is released */
            sm103::mma_commit(drain);
            uint64_t t0 = sm103::globaltimer();
            while (!sm103::mbar_try_wait(drain, 0) && sm103::globaltimer() - t0 < sm103::kWaitLimitNs) {}
        }
    } else {
        /* ---------------- epilogue warps ---------------- */
        const int quarter = warp % 4;                  /* TMEM lane quarter this warp may access */
        const int colbase = ((warp - 2) / 4) * kEpiCols;
        const int row = quarter * 32 + lane;
        const uint32_t tl = tmem + ((uint32_t)(quarter * 32) << 16);
        int buf = 0;
        uint32_t aph = 0;
        bool ok = true;
        /* Z lines stay in L2 between the level folds of an item (evict_last);
         * the last fold marks them evict_first, as the GEMM is done with them */
        uint64_t pol_keep, pol_drop;
        asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol_keep));
        asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol_drop));
        ItemRing ring{sm103::smem_u32(sfull), 0, 0};
        for (;;) {
            int b;
            if (!ring.take_warp(&b, lane, abort_flag, L.err, 9)) { ok = false; break; }
            if (b < 0) break;
            const Item it = decode_item(L, b);
            const GemmProblem& P = L.prob[it.p];
            const int s = P.s, nkb = P.nkb;
            int64_t* zrow = P.Z + (int64_t)it.r * P.n_pad * P.m_pad +
                            (int64_t)(it.tile_n * kTileN + colbase) * P.m_pad + it.tile_m * kTileM + row;
            const struct { int zlevel, m_pad, db; } a = {P.zlevel, P.m_pad, P.db};
            for (int g = 2; g <= s + 1 && ok; ++g) {
                int lsum[kEpiCols];
#pragma unroll
                for (int x = 0; x < kEpiCols; ++x) lsum[x] = 0;
                const int nchunks = (level_pairs(g, s) * nkb + kChunkKB - 1) / kChunkKB;
                for (int c = 0; c < nchunks; ++c) {
                    if (!sm103::mbar_wait(&accf[buf], aph, abort_flag, L.err, 4)) { ok = false; break; }
                    sm103::tc_fence_after();
#pragma unroll
                    for (int h = 0; h < kEpiCols / 8; ++h) {
                        uint32_t v[8];
                        SM103_TMEM_LD_X8(tl + buf * kTileN + colbase + h * 8, v);
                        sm103::tmem_wait_ld();
#pragma unroll
                        for (int x = 0; x < 8; ++x)
                            lsum[h * 8 + x] += __float2int_rn(__uint_as_float(v[x]));   /* exact: integer, |v| <= 2^24 */
                    }
                    sm103::tc_fence_before();
                    __syncwarp();
                    if (lane == 0) sm103::mbar_arrive(&acce[buf]);
                    buf ^= 1;
                    if (buf == 0) aph ^= 1;
                }
                if (!ok) break;
                /* fold L_g into the Z tile (units of level G): D = G - g, exact
                 * left shift by db*D for D >= 0, rounded right shift by -db*D
                 * (ties up) for D < 0. The first level stores; later levels add with
                 * fire-and-forget 64-bit reductions (two's-complement addition
                 * is exact and order-free), so the warps go straight back to
                 * draining the accumulator. */
                {
                    const int D = a.zlevel - g;
                    const uint32_t lsh = D >= 0 ? a.db * D : 0;
                    const uint32_t rsh = D >= 0 ? 0 : -a.db * D;
                    const uint64_t rnd = D >= 0 ? 0 : (1ull << (rsh - 1));
                    uint64_t zp = (uint64_t)zrow;
                    const uint64_t zstep = (uint64_t)a.m_pad * 8;
                    const uint64_t pol = g == s + 1 ? pol_drop : pol_keep;
                    if (g == 2) {
#pragma unroll
                        for (int x = 0; x < kEpiCols; ++x)
                            asm volatile("{\n\t.reg .b64 t;\n\t"
                                         "cvt.s64.s32 t, %1;\n\t"
                                         "shl.b64 t, t, %2;\n\t"
                                         "st.global.L2::cache_hint.u64 [%0], t, %4;\n\t"
                                         "add.u64 %0, %0, %3;\n\t}"
                                         : "+l"(zp) : "r"(lsum[x]), "r"(lsh), "l"(zstep), "l"(pol) : "memory");
                    } else {
#pragma unroll
                        for (int x = 0; x < kEpiCols; ++x)
                            asm volatile("{\n\t.reg .b64 t;\n\t"
                                         "cvt.s64.s32 t, %1;\n\t"
                                         "shl.b64 t, t, %2;\n\t"
                                         "add.s64 t, t, %4;\n\t"
                                         "shr.s64 t, t, %3;\n\t"
                                         "red.global.add.L2::cache_hint.u64 [%0], t, %6;\n\t"
                                         "add.u64 %0, %0, %5;\n\t}"
                                         : "+l"(zp) : "r"(lsum[x]), "r"(lsh), "r"(rsh), "l"(rnd), "l"(zstep), "l"(pol)
                                         : "memory");
                    }
                }
            }
        }
    }
    sm103::tc_fence_before();
    __syncthreads();
    sm103::tc_fence_after();
    if (warp == 1) sm103::tmem_dealloc(tmem, kTmemCols);
}

/* ---------------------------------------------------- CTA-pair GEMM ---- */

constexpr int kPairTileM = 256;                       /* rows of a pair tile (128 per CTA) */
constexpr int kPairMinRows = 1024;                    /* m_e from which single calls use pair tiles */
constexpr int kPairStages = 6;
constexpr int kPairRasterGroup = 6;                   /* pair-tile rows per raster band (1536 rows) */
std::atomic<int> g_pair_rows{kPairMinRows};           /* m_e from which GEMMs take pair tiles (host) */
constexpr uint32_t kPairHalfBytes = 128 * kBK * 2;    /* 16 KB: 128 rows of one 128-byte stage row */
constexpr uint32_t kPairStageBytes = 2 * kPairHalfBytes;
constexpr size_t kPairSmem = (size_t)kPairStages * kPairStageBytes + 1024 + 512;



/* The same GEMM as split_gemm_kernel with CTA pairs (clusters of two), with
 * work items drawn dynamically: the even CTA's producer takes the next item
 * from L.sched (atomicAdd) and writes it into both CTAs' item rings; every
 * other role reads the ring, so the clusters' items in flight stay
 * contiguous and share operand panels in L2 (a static round robin lets them
 * drift apart). A work item is a 256 x 256 tile of a product; each CTA loads its 128 rows of the A
 * slice tile and its 128-column half of the B slice tile (32 KB per stage
 * instead of 48 KB, so the L2 feeds each SM a third less per MMA and the
 * six-stage ring looks 50% further ahead), and the even CTA issues
 * tcgen05.mma cta_group::2 (M=256, N=256) into both CTAs' TMEM. Both CTAs'
 * stage loads complete on the even CTA's barrier (TMA cta_group::2); the MMA
 * commits arrive on both CTAs' stage and accumulator barriers; each CTA's epilogue drains its own 128 rows exactly
 * as in split_gemm_kernel and reports the buffer free to the even CTA. All
 * waits are bounded; the two cluster barriers (after barrier set-up, before
 * TMEM release) are reached by every thread of both CTAs. */
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kGemmThreads, 1)
split_gemm_pair_kernel(const __grid_constant__ GemmLaunch L)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* sA = smem;
    uint8_t* sB = smem + kPairStages * kPairHalfBytes;
    uint64_t* full = (uint64_t*)(smem + kPairStages * kPairStageBytes);
    uint64_t* empty = full + kPairStages;
    uint64_t* accf = empty + kPairStages;
    uint64_t* acce = accf + 2;
    uint64_t* drain = acce + 2;
    uint64_t* sfull = drain + 1;                  /* item ring: slot written */
    uint64_t* sempty = sfull + kSchedSlots;       /* item ring: slot read by every consumer (even CTA) */
    int* sitem = (int*)(sempty + kSchedSlots);
    uint32_t* tmem_slot = (uint32_t*)(sitem + kSchedSlots);
    volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const uint32_t rank = sm103::cluster_ctarank();

    if (threadIdx.x == 0) {
        for (int i = 0; i < kPairStages; ++i) {
            sm103::mbar_init(&full[i], 1);
            sm103::mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) { sm103::mbar_init(&accf[i], 1); sm103::mbar_init(&acce[i], 2 * kEpiWarps); }
        sm103::mbar_init(drain, 1);
        for (int i = 0; i < kSchedSlots; ++i) {
            sm103::mbar_init(&sfull[i], 1);
            sm103::mbar_init(&sempty[i], kSchedConsumers);
        }
        *abort_flag = 0;
        sm103::fence_mbar_init();
    }
    if (warp == 1) { sm103::tmem_alloc_pair(tmem_slot, kTmemCols); sm103::tmem_relinquish_pair(); }
    sm103::tc_fence_before();
    sm103::cluster_sync();   /* both CTAs' barriers exist before any remote arrive */
    sm103::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        /* ---------------- TMA producer (both CTAs) ---------------- */
        if (lane == 0) {
            int st = 0;
            uint32_t ph = 0;
            uint32_t armed = 0;
            bool ok = true;
            int last_p = -1;
            ItemRing ring{sm103::smem_u32(sfull), 0, 0};
            for (;;) {
                int b;
                if (rank == 0) {
                    /* the even producer takes the next item and publishes it
                     * to both CTAs' rings */
                    if (!sm103::mbar_wait_acq_cluster_u32(ring.empty_at(), ring.ph ^ 1, abort_flag, L.err, 17)) {
                        ok = false;
                        break;
                    }
                    b = (int)atomicAdd(L.sched, 1u);
                    if (b >= L.nitems) b = -1;
                    sitem[ring.slot] = b;
                    sm103::st_shared_cluster_u32(sm103::mapa(sm103::smem_u32(&sitem[ring.slot]), 1), (uint32_t)b);
                    sm103::mbar_arrive(&sfull[ring.slot]);
                    sm103::mbar_arrive_release_cluster(sm103::mapa(sm103::smem_u32(&sfull[ring.slot]), 1));
                    ring.next();
                } else if (!ring.take(&b, abort_flag, L.err, 18)) {
                    ok = false;
                    break;
                }
                if (b < 0) break;
                const Item it = decode_item(L, b, kPairRasterGroup);
                const GemmProblem& P = L.prob[it.p];
                if (it.p != last_p) { sm103::prefetch_tmap(&P.tmA); sm103::prefetch_tmap(&P.tmB); last_p = it.p; }
                const int s = P.s, nkb = P.nkb;
                const int arow = it.r * s * P.m_pad + it.tile_m * kPairTileM + 128 * (int)rank;
                const int brow = it.r * s * P.n_pad + it.tile_n * kTileN + 128 * (int)rank;
                int pi = 0;   /* the single-CTA kernel's pair order */
                for (int g = 2; g <= s + 1 && ok; ++g) {
                    const int tlo = max(1, g - s), thi = min(s, g - 1);
                    for (int x = 0; x <= thi - tlo && ok; ++x, ++pi) {
                        const int t = (g & 1) ? thi - x : tlo + x;
                        const int u = g - t;
                        for (int y = 0; y < nkb; ++y) {
                            const int kb = (pi & 1) ? nkb - 1 - y : y;
                            if (!sm103::mbar_wait(&empty[st], ph ^ 1, abort_flag, L.err, 11)) { ok = false; break; }
                            /* both CTAs' loads complete on the even CTA's full[st]; the
                             * even CTA expects the bytes of both */
                            if (rank == 0) sm103::mbar_arrive_expect_tx(&full[st], 2 * kPairStageBytes);
                            const uint32_t fb = sm103::mapa(sm103::smem_u32(&full[st]), 0);
                            sm103::tma_load_2d_pair(sA + st * kPairHalfBytes, &P.tmA, fb, kb * P.kbe,
                                                    arow + (t - 1) * P.m_pad);
                            sm103::tma_load_2d_pair(sB + st * kPairHalfBytes, &P.tmB, fb, kb * P.kbe,
                                                    brow + (u - 1) * P.n_pad);
                            armed |= 1u << st;
                            if (++st == kPairStages) { st = 0; ph ^= 1; armed = 0; }
                        }
                    }
                }
            }
            if (!ok && rank == 0) {
                for (int i = 0; i < kPairStages; ++i) {
                    const uint32_t par = (armed >> i) & 1u ? ph : ph ^ 1;
                    uint64_t t0 = sm103::globaltimer();
                    while (!sm103::mbar_try_wait(&full[i], par) &&
                           sm103::globaltimer() - t0 < sm103::kWaitLimitNs) {}
                }
            }
            (void)armed;
        }
    } else if (warp == 1) {
        if (lane == 0 && rank == 0) {
            /* ---------------- even CTA: MMA issuer ---------------- */
            constexpr uint32_t idesc16 = sm103::idesc_bf16_f32(kPairTileM, kTileN);
            constexpr uint32_t idesc8 = sm103::idesc_e4m3_f32(kPairTileM, kTileN);
            int st = 0, buf = 0;
            uint32_t ph = 0, aph = 0;
            bool ok = true;
            ItemRing ring{sm103::smem_u32(sfull), 0, 0};
            for (;;) {
                int b;
                if (!ring.take(&b, abort_flag, L.err, 19)) { ok = false; break; }
                if (b < 0) break;
                const Item it = decode_item(L, b, kPairRasterGroup);
                const int s = L.prob[it.p].s, nkb = L.prob[it.p].nkb, fmt = L.prob[it.p].fmt;
                for (int g = 2; g <= s + 1 && ok; ++g) {
                    const int level_kb = level_pairs(g, s) * nkb;
                    for (int jl = 0; jl < level_kb && ok; ) {
                        if (jl % kChunkKB == 0) {
                            if (!sm103::mbar_wait(&acce[buf], aph ^ 1, abort_flag, L.err, 13)) { ok = false; break; }
                            sm103::tc_fence_after();
                        }
                        if (!sm103::mbar_wait(&full[st], ph, abort_flag, L.err, 14)) { ok = false; break; }
                        sm103::tc_fence_after();
                        const uint32_t a0 = sm103::smem_u32(sA + st * kPairHalfBytes);
                        const uint32_t b0 = sm103::smem_u32(sB + st * kPairHalfBytes);
                        if (fmt) {
#pragma unroll
                            for (int kk = 0; kk < 4; ++kk)
                                sm103::mma_f8_pair(tmem + buf * kTileN, sm103::smem_desc_sw128(a0 + kk * 32),
                                                   sm103::smem_desc_sw128(b0 + kk * 32), idesc8,
                                                   (jl % kChunkKB != 0 || kk != 0) ? 1u : 0u);
                        } else {
#pragma unroll
                            for (int kk = 0; kk < 4; ++kk)
                                sm103::mma_bf16_pair(tmem + buf * kTileN, sm103::smem_desc_sw128(a0 + kk * 32),
                                                     sm103::smem_desc_sw128(b0 + kk * 32), idesc16,
                                                     (jl % kChunkKB != 0 || kk != 0) ? 1u : 0u);
                        }
                        sm103::mma_commit_pair(&empty[st]);
                        if (++st == kPairStages) { st = 0; ph ^= 1; }
                        ++jl;
                        if (jl % kChunkKB == 0 || jl == level_kb) {
                            sm103::mma_commit_pair(&accf[buf]);
                            buf ^= 1;
                            if (buf == 0) aph ^= 1;
                        }
                    }
                }
            }
            /* all issued MMAs complete before either CTA releases TMEM */
            sm103::mma_commit_pair(drain);
            uint64_t t0 = sm103::globaltimer();
            while (!sm103::mbar_try_wait(drain, 0) && sm103::globaltimer() - t0 < sm103::kWaitLimitNs) {}
        }
    } else {
        /* ---------------- epilogue warps (both CTAs) ---------------- */
        const int quarter = warp % 4;
        const int colbase = ((warp - 2) / 4) * kEpiCols;
        const int row = quarter * 32 + lane;
        const uint32_t tl = tmem + ((uint32_t)(quarter * 32) << 16);
        const uint32_t acce0 = sm103::mapa(sm103::smem_u32(acce), 0);
        int buf = 0;
        uint32_t aph = 0;
        bool ok = true;
        uint64_t pol_keep, pol_drop;
        asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol_keep));
        asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol_drop));
        ItemRing ring{sm103::smem_u32(sfull), 0, 0};
        for (;;) {
            int b;
            if (!ring.take_warp(&b, lane, abort_flag, L.err, 20)) { ok = false; break; }
            if (b < 0) break;
            const Item it = decode_item(L, b, kPairRasterGroup);
            const GemmProblem& P = L.prob[it.p];
            const int s = P.s, nkb = P.nkb;
            int64_t* zrow = P.Z + (int64_t)it.r * P.n_pad * P.m_pad +
                            (int64_t)(it.tile_n * kTileN + colbase) * P.m_pad + it.tile_m * kPairTileM +
                            128 * (int)rank + row;
            const struct { int zlevel, m_pad, db; } a = {P.zlevel, P.m_pad, P.db};
            for (int g = 2; g <= s + 1 && ok; ++g) {
                int lsum[kEpiCols];
#pragma unroll
                for (int x = 0; x < kEpiCols; ++x) lsum[x] = 0;
                const int nchunks = (level_pairs(g, s) * nkb + kChunkKB - 1) / kChunkKB;
                for (int c = 0; c < nchunks; ++c) {
                    if (!sm103::mbar_wait(&accf[buf], aph, abort_flag, L.err, 16)) { ok = false; break; }
                    sm103::tc_fence_after();
#pragma unroll
                    for (int h = 0; h < kEpiCols / 8; ++h) {
                        uint32_t v[8];
                        SM103_TMEM_LD_X8(tl + buf * kTileN + colbase + h * 8, v);
                        sm103::tmem_wait_ld();
#pragma unroll
                        for (int x = 0; x < 8; ++x)
                            lsum[h * 8 + x] += __float2int_rn(__uint_as_float(v[x]));   /* exact: integer, |v| <= 2^24 */
                    }
                    sm103::tc_fence_before();
                    __syncwarp();
                    if (lane == 0) sm103::mbar_arrive_cluster(acce0 + buf * 8);
                    buf ^= 1;
                    if (buf == 0) aph ^= 1;
                }
                if (!ok) break;
                /* fold L_g into the Z tile, as in split_gemm_kernel */
                {
                    const int D = a.zlevel - g;
                    const uint32_t lsh = D >= 0 ? a.db * D : 0;
                    const uint32_t rsh = D >= 0 ? 0 : -a.db * D;
                    const uint64_t rnd = D >= 0 ? 0 : (1ull << (rsh - 1));
                    uint64_t zp = (uint64_t)zrow;
                    const uint64_t zstep = (uint64_t)a.m_pad * 8;
                    const uint64_t pol = g == s + 1 ? pol_drop : pol_keep;
                    if (g == 2) {
#pragma unroll
                        for (int x = 0; x < kEpiCols; ++x)
                            asm volatile("{\n\t.reg .b64 t;\n\t"
                                         "cvt.s64.s32 t, %1;\n\t"
                                         "shl.b64 t, t, %2;\n\t"
                                         "st.global.L2::cache_hint.u64 [%0], t, %4;\n\t"
                                         "add.u64 %0, %0, %3;\n\t}"
                                         : "+l"(zp) : "r"(lsum[x]), "r"(lsh), "l"(zstep), "l"(pol) : "memory");
                    } else {
#pragma unroll
                        for (int x = 0; x < kEpiCols; ++x)
                            asm volatile("{\n\t.reg .b64 t;\n\t"
                                         "cvt.s64.s32 t, %1;\n\t"
                                         "shl.b64 t, t, %2;\n\t"
                                         "add.s64 t, t, %4;\n\t"
                                         "shr.s64 t, t, %3;\n\t"
                                         "red.global.add.L2::cache_hint.u64 [%0], t, %6;\n\t"
                                         "add.u64 %0, %0, %5;\n\t}"
                                         : "+l"(zp) : "r"(lsum[x]), "r"(lsh), "r"(rsh), "l"(rnd), "l"(zstep), "l"(pol)
                                         : "memory");
                    }
                }
            }
        }
    }
    sm103::tc_fence_before();
    __syncthreads();
    sm103::cluster_sync();   /* no remote arrive or MMA still targets either CTA */
    sm103::tc_fence_after();
    if (warp == 1) sm103::tmem_dealloc_pair(tmem, kTmemCols);
}

/* Multi-C epilogue for a group of products [r0, r0 + nprod): one thread per
 * (C sub-block p = blockIdx.y, element (i, j) of p) adds alpha*W[p,r] *
 * M_r[i,j] for the group's products in increasing order, with M_r[i,j] =
 * 2^(E_i + F_j + 2 - db*G) * Z_r[i,j] = 2^(ebase + E_i + F_j) * Z_r[i,j]
 * converted in integer arithmetic
 * (plugin/ref_kernels/bli_gemm_fmm_ref.c:99-120, once per group instead of
 * once per product). */
constexpr int kScatterMaxEnt = 1024;

__global__ void __launch_bounds__(256)
scatter_kernel(const int* __restrict__ tab, int r0, int nprod, int64_t m, int64_t n,
               int m_pad, int n_pad, int ebase, double alpha, const int64_t* __restrict__ Z,
               const int* __restrict__ e_row, const int* __restrict__ f_col, double* __restrict__ C,
               int64_t ldc)
{
    __shared__ double lam[kScatterMaxEnt];
    __shared__ int prod[kScatterMaxEnt];
    __shared__ int nsel;
    const Tab t = tab_view(tab);
    const int p = blockIdx.y;
    int ro, rl, co, cl;
    fmm_part_geom32((int)m, t.mt, p / t.nt, &ro, &rl);
    fmm_part_geom32((int)n, t.nt, p % t.nt, &co, &cl);
    if (rl <= 0 || cl <= 0) return;   /* empty sub-block (dimension smaller than its split) */
    /* this part's entries that fall in the group, in product order */
    if (threadIdx.x == 0) {
        int q = 0;
        for (int e = t.wp_off[p]; e < t.wp_off[p + 1] && q < kScatterMaxEnt; ++e) {
            const int r = t.wp_ent[2 * e] - r0;
            if (r < 0) continue;
            if (r >= nprod) break;
            prod[q] = r;
            lam[q] = alpha * (double)t.wp_ent[2 * e + 1];
            ++q;
        }
        nsel = q;
    }
    __syncthreads();
    const int ne = nsel;
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (ne == 0 || idx >= (uint32_t)rl * (uint32_t)cl) return;
    const int i = (int)(idx % (uint32_t)rl), j = (int)(idx / (uint32_t)rl);
    double* cp = C + ro + i + (int64_t)(co + j) * ldc;
    double c = *cp;
    const int64_t zij = (int64_t)j * m_pad + i;
    const int64_t zstride = (int64_t)n_pad * m_pad;
    int q = 0;
    for (; q + 4 <= ne; q += 4) {
        int64_t z[4];
        int ex[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int r = prod[q + u];
            z[u] = Z[r * zstride + zij];
            ex[u] = e_row[r * m_pad + i] + f_col[r * n_pad + j] + ebase;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) c = fma(lam[q + u], i64_to_double_scaled(z[u], ex[u]), c);
    }
    for (; q < ne; ++q) {
        const int r = prod[q];
        c = fma(lam[q], i64_to_double_scaled(Z[r * zstride + zij], e_row[r * m_pad + i] + f_col[r * n_pad + j] + ebase), c);
    }
    *cp = c;
}

/* one element (i, j) of the product grid for scatter_all_kernel */
__device__ __forceinline__ void scatter_all_element(uint64_t idx, uint32_t rows, uint32_t i_lo, int P, int T, int tid,
                                                    int nprod,
                                                    int m_pad, int n_pad, int ebase, const int (&geo)[4][64],
                                                    double* cs, const double* lam, const int* pidx, const int* off,
                                                    const int64_t* __restrict__ Z, const int* __restrict__ e_row,
                                                    const int* __restrict__ f_col, double* __restrict__ C,
                                                    int64_t ldc)
{
    const int i = (int)(i_lo + (uint32_t)idx % rows), j = (int)((uint32_t)idx / rows);
    uint64_t live = 0;
    for (int p = 0; p < P; ++p) {
        if (i < geo[1][p] && j < geo[3][p]) {
            live |= 1ull << p;
            cs[p * T + tid] = C[geo[0][p] + i + (int64_t)(geo[2][p] + j) * ldc];
        }
    }
    const int64_t zij = (int64_t)j * m_pad + i;
    const int64_t zstride = (int64_t)n_pad * m_pad;
    int q = 0;
    for (; q + 4 <= nprod; q += 4) {
        int64_t z[4];
        int ex[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            z[u] = Z[(q + u) * zstride + zij];
            ex[u] = e_row[(int64_t)(q + u) * m_pad + i] + f_col[(int64_t)(q + u) * n_pad + j] + ebase;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int b = off[q + u], e = off[q + u + 1];
            if (b == e) continue;
            const double M = i64_to_double_scaled(z[u], ex[u]);
            for (int x = b; x < e; ++x) {
                const int p = pidx[x];
                if ((live >> p) & 1ull) cs[p * T + tid] = fma(lam[x], M, cs[p * T + tid]);
            }
        }
    }
    for (; q < nprod; ++q) {
        const int b = off[q], e = off[q + 1];
        if (b == e) continue;
        const double M = i64_to_double_scaled(Z[q * zstride + zij],
                                              e_row[(int64_t)q * m_pad + i] + f_col[(int64_t)q * n_pad + j] + ebase);
        for (int x = b; x < e; ++x) {
            const int p = pidx[x];
            if ((live >> p) & 1ull) cs[p * T + tid] = fma(lam[x], M, cs[p * T + tid]);
        }
    }
    for (int p = 0; p < P; ++p)
        if ((live >> p) & 1ull) C[geo[0][p] + i + (int64_t)(geo[2][p] + j) * ldc] = cs[p * T + tid];
}

/* Multi-C epilogue, element-major: one thread per element (i, j) of the
 * product grid (element index i + j*m_e in [idx_first, idx_end), grid-stride)
 * updates that element of every C sub-block p, so each product's
 * Z_r[i,j] is read and converted once and shared by all sub-blocks it feeds.
 * The sub-blocks' running values live in shared memory (cs[p][thread]); for
 * every sub-block the updates still come in increasing product order, so the
 * result is identical to scatter_kernel's. Used when the sub-block count and
 * the group's W entries fit the shared-memory budget. */
constexpr int kScatterAllSmem = 32 * 1024;   /* cs[] budget: P * threads * 8 */

/* vb, vg: the block's index among the vg blocks that share the element range */
__device__ __forceinline__ void scatter_all_body(const int* __restrict__ tab, int r0, int nprod, int64_t m, int64_t n,
                                                 int m_pad, int n_pad, int ebase, double alpha,
                                                 const int64_t* __restrict__ Z, const int* __restrict__ e_row,
                                                 const int* __restrict__ f_col, double* __restrict__ C, int64_t ldc,
                                                 uint64_t idx_first, uint64_t idx_end, uint64_t vb, uint64_t vg,
                                                 uint32_t i_lo = 0, uint32_t i_rows = 0)
{
    extern __shared__ double sm_all[];
    __shared__ int geo[4][64];           /* per sub-block p: ro, rl, co, cl */
    const Tab t = tab_view(tab);
    const int P = t.mt * t.nt, T = (int)blockDim.x, tid = (int)threadIdx.x;
    const int eb = t.w_off[r0], E = t.w_off[r0 + nprod] - eb;
    double* cs = sm_all;                 /* [P][T] */
    double* lam = cs + (size_t)P * T;    /* [E] */
    int* pidx = (int*)(lam + E);         /* [E] */
    int* off = pidx + E;                 /* [nprod + 1] */
    for (int x = tid; x < E; x += T) {
        pidx[x] = t.w_ent[2 * (eb + x)];
        lam[x] = alpha * (double)t.w_ent[2 * (eb + x) + 1];
    }
    for (int x = tid; x <= nprod; x += T) off[x] = t.w_off[r0 + x] - eb;
    for (int p = tid; p < P; p += T) {
        fmm_part_geom32((int)m, t.mt, p / t.nt, &geo[0][p], &geo[1][p]);
        fmm_part_geom32((int)n, t.nt, p % t.nt, &geo[2][p], &geo[3][p]);
    }
    __syncthreads();
    const uint32_t me = (uint32_t)((m + t.mt - 1) / t.mt), ne = (uint32_t)((n + t.nt - 1) / t.nt);
    /* the product-grid rows [i_lo, i_lo + rows) of every column, element
     * index (i - i_lo) + j * rows (all rows when i_rows is 0); rows * ne <
     * 2^32 (checked on the host), so the element index fits 32 bits */
    const uint32_t rows = i_rows ? i_rows : me;
    const uint64_t idx = idx_first + vb * (uint64_t)T + (uint64_t)tid;
    const uint64_t end = idx_end < (uint64_t)rows * (uint64_t)ne ? idx_end : (uint64_t)rows * (uint64_t)ne;
    if (P == 1 && E == 1 && nprod == 1) {
        /* one sub-block fed by one product (the classical split GEMM): the
         * same conversion and FMA per element without the per-sub-block
         * bookkeeping, the element's C value kept in a register */
        const double l = lam[0];
        const uint64_t step = vg * (uint64_t)T;
        constexpr int U = 2;   /* elements per thread per round: their loads go out together */
        const int ro = geo[0][0], rl = geo[1][0], co = geo[2][0], cl = geo[3][0];
        for (uint64_t idx2 = idx; idx2 < end; idx2 += U * step) {
            int64_t z[U];
            int ex[U];
            double c[U];
            int ii[U], jj[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint64_t e = idx2 + u * step;
                ii[u] = (int)(i_lo + (uint32_t)e % rows);
                jj[u] = e < end ? (int)((uint32_t)e / rows) : cl;   /* past the end: not live */
                z[u] = 0;
                ex[u] = 0;
                c[u] = 0.0;
                if (ii[u] < rl && jj[u] < cl) {
                    z[u] = Z[(int64_t)jj[u] * m_pad + ii[u]];
                    ex[u] = e_row[ii[u]] + f_col[jj[u]] + ebase;
                    c[u] = C[ro + ii[u] + (int64_t)(co + jj[u]) * ldc];
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (ii[u] < rl && jj[u] < cl)
                    C[ro + ii[u] + (int64_t)(co + jj[u]) * ldc] = fma(l, i64_to_double_scaled(z[u], ex[u]), c[u]);
        }
        return;
    }
    /* grid-stride: a block's set-up above serves many elements */
    for (uint64_t idx2 = idx; idx2 < end; idx2 += vg * (uint64_t)T)
        scatter_all_element(idx2, rows, i_lo, P, T, tid, nprod, m_pad, n_pad, ebase, geo, cs, lam, pidx, off, Z,
                            e_row, f_col, C, ldc);
}

__global__ void __launch_bounds__(256)
scatter_all_kernel(const int* __restrict__ tab, int r0, int nprod, int64_t m, int64_t n,
                   int m_pad, int n_pad, int ebase, double alpha, const int64_t* __restrict__ Z,
                   const int* __restrict__ e_row, const int* __restrict__ f_col, double* __restrict__ C,
                   int64_t ldc, uint64_t idx_first, uint64_t idx_end, uint32_t i_lo, uint32_t i_rows)
{
    scatter_all_body(tab, r0, nprod, m, n, m_pad, n_pad, ebase, alpha, Z, e_row, f_col, C, ldc, idx_first, idx_end,
                     blockIdx.x, gridDim.x, i_lo, i_rows);
}


/* ------------------------------------- batched waves: side work per wave ---- */

/* A wave of a batch runs each side kernel (C scaling and maxima zeroing,
 * maxima, exponents, packs, C updates) as one launch over all its problems
 * instead of one launch per problem: the problems travel by value in a table
 * (like the GEMM's), each owns a contiguous range of the launch's blocks, and
 * a block finds its problem by binary search and runs the same per-block code
 * (the *_body functions) the single-problem kernels run, so the results are
 * the single calls' bits. */
struct WaveProb {
    const int* tab;
    const double* A;
    const double* B;
    double* C;
    unsigned long long* amax;
    unsigned long long* bmax;
    int* e_row;
    int* f_col;
    uint8_t* sa;
    uint8_t* sb;
    const int64_t* Z;
    int64_t lda, ldb, ldc, m, n, k, m_pad, n_pad, k_pad;
    int64_t b0;   /* the problem's first block in this launch */
    int64_t nb;   /* its blocks */
    int64_t gx;   /* blocks along the first coordinate of its per-problem grid */
    double alpha, beta;
    int R, kt, ebase;
};
struct WaveLaunch {
    int nprob;
    WaveProb p[kMaxLaunchProblems];
};
static_assert(sizeof(WaveLaunch) <= 32764, "WaveLaunch must fit the kernel parameter space");

__device__ __forceinline__ int wave_find(const WaveLaunch& W, int64_t b)
{
    int lo = 0, hi = W.nprob - 1;   /* last problem with b0 <= b */
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (W.p[mid].b0 <= b) lo = mid; else hi = mid - 1;
    }
    return lo;
}

/* C := beta*C (when beta != 1) and the maxima arrays zeroed, grid-stride over each problem's range */
__global__ void __launch_bounds__(256) wave_prep_kernel(const __grid_constant__ WaveLaunch W)
{
    const WaveProb& P = W.p[wave_find(W, blockIdx.x)];
    const int64_t vb = blockIdx.x - P.b0;
    const int64_t za = (int64_t)P.kt * P.m, zb = (int64_t)P.kt * P.n;
    const int64_t total = za + zb + (P.beta != 1.0 ? P.m * P.n : 0);
    for (int64_t x = vb * blockDim.x + threadIdx.x; x < total; x += P.nb * (int64_t)blockDim.x) {
        if (x < za) {
            P.amax[x] = 0;
        } else if (x < za + zb) {
            P.bmax[x - za] = 0;
        } else {
            const int64_t e = x - za - zb;
            double* c = P.C + e % P.m + (e / P.m) * P.ldc;
            *c = P.beta == 0.0 ? 0.0 : P.beta * *c;
        }
    }
}

/* row maxima of A (gx blocks: 256 rows x one k part x 256 columns) then column maxima of B */
__global__ void __launch_bounds__(256) wave_maxima_kernel(const __grid_constant__ WaveLaunch W)
{
    const WaveProb& P = W.p[wave_find(W, blockIdx.x)];
    const int64_t vb = blockIdx.x - P.b0;
    if (vb < P.gx) {
        const int64_t rb = (P.m + 255) / 256;
        amax_body(P.A, P.lda, P.m, P.k, P.kt, P.amax, 256, vb % rb, (int)((vb / rb) % P.kt), vb / rb / P.kt);
    } else {
        bmax_body(P.B, P.ldb, P.k, P.n, P.kt, P.bmax, 0, P.n, vb - P.gx);
    }
}

__global__ void __launch_bounds__(256) wave_exps_kernel(const __grid_constant__ WaveLaunch W)
{
    const WaveProb& P = W.p[wave_find(W, blockIdx.x)];
    const int64_t vb = blockIdx.x - P.b0;
    exps_body(P.tab, 0, P.m, P.n, P.k, P.m_pad, P.n_pad, P.amax, P.bmax, P.e_row, P.f_col, 0, P.m_pad + P.n_pad,
              vb % P.gx, (int)(vb / P.gx));
}

template <int S, int DB, int ROWS>
__global__ void __launch_bounds__(ROWS * 4, ROWS == 64 ? 4 : 8) wave_pack_a_kernel(const __grid_constant__ WaveLaunch W)
{
    const WaveProb& P = W.p[wave_find(W, blockIdx.x)];
    const int64_t vb = blockIdx.x - P.b0;
    pack_a_body<S, DB, ROWS>(P.tab, 0, P.R, P.A, P.lda, P.m, P.k, P.m_pad, P.k_pad, P.e_row, P.sa, vb % P.gx,
                             vb / P.gx);
}

template <int S, int DB, int COLS>
__global__ void __launch_bounds__(COLS * 8, COLS == 32 ? 4 : 8) wave_pack_b_kernel(const __grid_constant__ WaveLaunch W)
{
    const WaveProb& P = W.p[wave_find(W, blockIdx.x)];
    const int64_t vb = blockIdx.x - P.b0;
    pack_b_body<S, DB, COLS>(P.tab, 0, P.R, P.B, P.ldb, P.k, P.n, P.n_pad, P.k_pad, P.f_col, P.sb, 0, vb % P.gx,
                             vb / P.gx);
}

__global__ void __launch_bounds__(256) wave_scatter_kernel(const __grid_constant__ WaveLaunch W)
{
    const WaveProb& P = W.p[wave_find(W, blockIdx.x)];
    const int64_t vb = blockIdx.x - P.b0;
    const Tab t = tab_view(P.tab);
    const uint64_t me = (uint64_t)((P.m + t.mt - 1) / t.mt), ne = (uint64_t)((P.n + t.nt - 1) / t.nt);
    scatter_all_body(P.tab, 0, P.R, P.m, P.n, (int)P.m_pad, (int)P.n_pad, P.ebase, P.alpha, P.Z, P.e_row, P.f_col,
                     P.C, P.ldc, 0, me * ne, (uint64_t)vb, (uint64_t)P.nb);
}

/* --------------------------------------------------------- host -------- */

PFN_cuTensorMapEncodeTiled_v12000 get_encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, []() {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    });
    return fn;
}

/* 2-D map over slices[rows_total][k_pad] of BF16 (fmt 0) or FP8-E4M3 bytes
 * (fmt 1): boxes one 128-byte row of k (64 or 128 elements) by box_rows rows,
 * 128-byte swizzle. */
int make_slice_map(CUtensorMap* map, const void* base, int64_t k_pad, int64_t rows_total, int box_rows, int fmt)
{
    PFN_cuTensorMapEncodeTiled_v12000 enc = get_encode_fn();
    if (!enc) return FMM_ERR_CUDA;
    const int esz = fmt ? 1 : 2;                         /* FP8-E4M3 bytes or BF16 */
    cuuint64_t dims[2] = {(cuuint64_t)k_pad, (cuuint64_t)rows_total};
    cuuint64_t strides[1] = {(cuuint64_t)(k_pad * esz)};
    cuuint32_t box[2] = {(cuuint32_t)(128 / esz), (cuuint32_t)box_rows};   /* 128-byte rows */
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, fmt ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                     const_cast<void*>(base), dims, strides, box,
                     estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? FMM_OK : FMM_ERR_CUDA;
}

/* Products are processed in groups: all products of a group are packed, then
 * one GEMM launch covers every (product, tile) work item of the group, then
 * one scatter pass updates C. The group size is the largest that keeps the
 * per-group workspace (slices + Z) under kGroupBudget. */
constexpr size_t kGroupBudget = (size_t)32 << 30;

struct Dims {
    int64_t me, ne, ke, m_pad, n_pad, k_pad;
};

/* k elements per 128-byte stage row of a slice format */
inline int kbe_of(int fmt) { return fmt ? 128 : kBK; }

Dims dims_of(const AlgView& alg, int64_t m, int64_t n, int64_t k, int fmt = 0)
{
    Dims d;
    d.me = (m + alg.mt - 1) / alg.mt;
    d.ne = (n + alg.nt - 1) / alg.nt;
    d.ke = (k + alg.kt - 1) / alg.kt;
    /* rows padded to the 256-row pair tiles once m_e >= 1024 (at most 25%
     * padding there); any multiple of 128 also serves the single-CTA kernel */
    d.m_pad = round_up(std::max<int64_t>(d.me, 1), d.me >= kPairMinRows ? kPairTileM : kTileM);
    d.n_pad = round_up(std::max<int64_t>(d.ne, 1), kTileN);
    d.k_pad = round_up(std::max<int64_t>(d.ke, 1), kbe_of(fmt));
    return d;
}

size_t per_product_bytes(const Dims& d, int s, int fmt)
{
    return (fmt ? 1 : 2) * (size_t)s * (size_t)(d.m_pad + d.n_pad) * (size_t)d.k_pad +
           8 * (size_t)d.m_pad * (size_t)d.n_pad + 4 * (size_t)(d.m_pad + d.n_pad) + 1024;
}

int group_size(const AlgView& alg, const Dims& d, int s, size_t budget, int fmt)
{
    const size_t per = per_product_bytes(d, s, fmt);
    size_t g = budget / per;
    if (g < 1) g = 1;
    if (g > (size_t)alg.R) g = (size_t)alg.R;
    /* tensor-map row coordinates are 32-bit */
    while (g > 1 && (int64_t)g * s * std::max(d.m_pad, d.n_pad) > 0x7fffffffLL) --g;
    return (int)g;
}

struct WsLayout {
    size_t amax, bmax, sched, erow, fcol, sa, sb, z, total;
    int group;
};

WsLayout ws_layout_g(const AlgView& alg, const Dims& d, int64_t m, int64_t n, int s, int G, int fmt)
{
    const size_t esz = fmt ? 1 : 2;
    WsLayout L;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) / 256 * 256; return o; };
    L.group = G;
    L.amax = take(sizeof(unsigned long long) * (size_t)alg.kt * (size_t)m);
    L.bmax = take(sizeof(unsigned long long) * (size_t)alg.kt * (size_t)n);
    L.sched = take(sizeof(unsigned int));   /* the pair GEMM's work-item counter */
    L.erow = take(sizeof(int) * (size_t)G * (size_t)d.m_pad);
    L.fcol = take(sizeof(int) * (size_t)G * (size_t)d.n_pad);
    L.sa = take(esz * (size_t)G * s * (size_t)d.m_pad * (size_t)d.k_pad);
    L.sb = take(esz * (size_t)G * s * (size_t)d.n_pad * (size_t)d.k_pad);
    L.z = take(8 * (size_t)G * (size_t)d.m_pad * (size_t)d.n_pad);
    L.total = off;
    return L;
}

/* Layout for the largest product group whose whole workspace fits in
 * `budget` bytes (at least one product). */
WsLayout ws_layout(const AlgView& alg, int64_t m, int64_t n, int64_t k, int s, size_t budget = kGroupBudget,
                   int fmt = 0)
{
    const Dims d = dims_of(alg, m, n, k, fmt);
    int G = group_size(alg, d, s, budget, fmt);
    WsLayout L = ws_layout_g(alg, d, m, n, s, G, fmt);
    while (G > 1 && L.total > budget) L = ws_layout_g(alg, d, m, n, s, --G, fmt);
    return L;
}

/* opt-in event timing of the GEMM launches */
std::mutex g_timing_mu;
bool g_timing = false;
std::vector<std::pair<cudaEvent_t, cudaEvent_t>> g_pending, g_pool;
uint64_t g_timed_products = 0;

void timing_mark(cudaStream_t st, bool before)
{
    static thread_local std::pair<cudaEvent_t, cudaEvent_t> cur;
    std::lock_guard<std::mutex> lk(g_timing_mu);
    if (before) {
        if (g_pool.empty()) {
            cudaEvent_t a, b;
            cudaEventCreate(&a);
            cudaEventCreate(&b);
            g_pool.push_back({a, b});
        }
        cur = g_pool.back();
        g_pool.pop_back();
        cudaEventRecord(cur.first, st);
    } else {
        cudaEventRecord(cur.second, st);
        g_pending.push_back(cur);
    }
}

}  // namespace

extern "C" int fmm_gpu_set_split_pair_rows(int min_rows)
{
    return g_pair_rows.exchange(std::max(min_rows, kPairMinRows));
}

extern "C" void fmm_gpu_set_kernel_timing(int enable)
{
    std::lock_guard<std::mutex> lk(g_timing_mu);
    g_timing = enable != 0;
}

extern "C" int fmm_gpu_read_kernel_timing(double* total_ms, uint64_t* launches, uint64_t* products)
{
    std::lock_guard<std::mutex> lk(g_timing_mu);
    double sum = 0.0;
    int rc = FMM_OK;
    for (auto& pr : g_pending) {
        float ms = 0.f;
        if (cudaEventSynchronize(pr.second) != cudaSuccess ||
            cudaEventElapsedTime(&ms, pr.first, pr.second) != cudaSuccess)
            rc = FMM_ERR_CUDA;
        sum += ms;
        g_pool.push_back(pr);
    }
    if (launches) *launches = g_pending.size();
    if (products) *products = g_timed_products;
    if (total_ms) *total_ms = sum;
    g_pending.clear();
    g_timed_products = 0;
    return rc;
}

size_t fmm_split_ws_bytes(const AlgView& alg, int64_t m, int64_t n, int64_t k, int slices, int fmt)
{
    const WsLayout L = ws_layout(alg, m, n, k, slices, kGroupBudget, fmt);
    if (L.group < alg.R) return L.total;
    /* room for the two overlapping product groups when they fit the budget */
    const Dims d = dims_of(alg, m, n, k, fmt);
    const int G1 = (alg.R + 1) / 2;
    if (alg.R < 2) return L.total;
    const WsLayout L1 = ws_layout_g(alg, d, m, n, slices, G1, fmt);
    const size_t two = L1.total + (L1.total - L1.erow);
    return two <= kGroupBudget ? std::max(L.total, two) : L.total;
}

/* One split-form GEMM problem being executed: its algorithm, geometry,
 * operands and the part of the workspace it uses. */
struct SplitJob {
    AlgView alg;
    Dims d;
    int64_t m, n, k;
    double alpha, beta;
    const double* A;
    int64_t lda;
    const double* B;
    int64_t ldb;
    double* C;
    int64_t ldc;
    int s;
    int fmt;       /* 0: BF16 slices, 1: FP8-E4M3 slices */
    bool trivial;  /* nothing beyond C := beta*C */
    WsLayout L;
    uint8_t* w;
};

static int job_init(SplitJob& j, const AlgView& alg, int64_t m, int64_t n, int64_t k, double alpha,
                    const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C,
                    int64_t ldc, int s, int fmt = 0)
{
    if (fmt != 0 && fmt != 1) return FMM_ERR_ARG;
    if (s < 2 || s > (fmt ? 12 : 8)) return FMM_ERR_ARG;
    j.fmt = fmt;
    j.alg = alg;
    j.m = m; j.n = n; j.k = k;
    j.alpha = alpha; j.beta = beta;
    j.A = A; j.lda = lda; j.B = B; j.ldb = ldb; j.C = C; j.ldc = ldc;
    j.s = s;
    j.w = nullptr;
    j.trivial = m == 0 || n == 0 || k == 0 || alpha == 0.0;
    if (j.trivial) return FMM_OK;
    if (alg.max_nnz_u > kPackMaxEnt || alg.max_nnz_v > kPackMaxEnt) return FMM_ERR_UNSUPPORTED;
    if (m > 0x7fffffffLL || n > 0x7fffffffLL) return FMM_ERR_UNSUPPORTED;
    j.d = dims_of(alg, m, n, k, fmt);
    if (j.d.ke > kMaxKe) return FMM_ERR_UNSUPPORTED;
    if (j.d.me * j.d.ne > 0xffffffffLL) return FMM_ERR_UNSUPPORTED;
    /* the scatter keeps one C part's W entries of a group in shared memory */
    const Tab ht = tab_view(alg.htab);
    for (int p = 0; p < alg.mt * alg.nt; ++p)
        if (ht.wp_off[p + 1] - ht.wp_off[p] > kScatterMaxEnt) return FMM_ERR_UNSUPPORTED;
    return FMM_OK;
}

/* workspace of the job for a product group within `budget` bytes */
static int job_bind(SplitJob& j, void* ws, size_t ws_bytes, size_t budget)
{
    if (j.trivial) return FMM_OK;
    j.L = ws_layout(j.alg, j.m, j.n, j.k, j.s, budget, j.fmt);
    if ((int64_t)j.L.group * j.s * std::max(j.d.m_pad, j.d.n_pad) > 0x7fffffffLL) return FMM_ERR_UNSUPPORTED;
    if (ws == nullptr || ws_bytes < j.L.total) return FMM_ERR_WORKSPACE;
    if (((uintptr_t)ws & 255) != 0) return FMM_ERR_ARG;
    j.w = (uint8_t*)ws;
    return FMM_OK;
}

/* workspace of the job for a group of exactly G products */
static int job_bind_group(SplitJob& j, void* ws, size_t ws_bytes, int G)
{
    if (j.trivial) return FMM_OK;
    j.L = ws_layout_g(j.alg, j.d, j.m, j.n, j.s, G, j.fmt);
    if ((int64_t)j.L.group * j.s * std::max(j.d.m_pad, j.d.n_pad) > 0x7fffffffLL) return FMM_ERR_UNSUPPORTED;
    if (ws == nullptr || ws_bytes < j.L.total) return FMM_ERR_WORKSPACE;
    if (((uintptr_t)ws & 255) != 0) return FMM_ERR_ARG;
    j.w = (uint8_t*)ws;
    return FMM_OK;
}

/* Side streams: in a batch wave, the per-problem work (maxima, exponents,
 * packs, scatter) of different problems, so their small kernels overlap
 * instead of queueing behind each other on the caller's stream; in a single
 * call, the B-side maxima and pack beside the A-side ones. Created once per
 * device; forked from and joined back to the caller's stream with events,
 * which a stream capture follows. One call at a time uses a pool (g_side_use). */
/* Timeline of the last host-buffer call (fmm_gpu_set_host_timeline): device
 * times, from the first copy's start, of A on the device, B on the device,
 * the first GEMM launch's start, the last GEMM launch's end, C's last column
 * chunk back on the host; plus the call's host wall time. */
constexpr int kTimelinePoints = 5;
std::atomic<bool> g_timeline{false};
std::mutex g_timeline_mu;
double g_timeline_ms[kTimelinePoints + 1] = {0, 0, 0, 0, 0, 0};

constexpr int kWaveStreams = 8;                  /* batched waves: pack streams, then scatter streams */
constexpr int kSideStreams = 2 * kWaveStreams;

struct SidePool {
    int device;
    cudaStream_t s[kSideStreams];
    cudaEvent_t fork;
    cudaEvent_t join[kSideStreams];
    cudaEvent_t wave_pk[2][kWaveStreams];   /* a workspace half's packs done */
    cudaEvent_t wave_gm[2];                 /* a workspace half's GEMM done */
    cudaEvent_t wave_sc[2][kWaveStreams];   /* a workspace half's C updates done */
    cudaEvent_t gate[3];   /* host-buffer calls: A, B and C on the device */
    cudaEvent_t chunk[32]; /* host-buffer calls: B chunks in (0..7), C chunks out (8..31) */
    cudaEvent_t blk[10];   /* host-buffer calls, blocked schedule: A halves up, A and B halves packed, GEMM blocks done */
    cudaEvent_t tl[kTimelinePoints + 1];  /* host-buffer calls: the call's timeline (timing events) */
    cudaStream_t hi;       /* greatest priority: GEMMs that side work runs beside */
};

std::mutex g_side_mu, g_side_use;
std::vector<SidePool*> g_side;

SidePool* side_pool()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(g_side_mu);
    for (SidePool* p : g_side)
        if (p->device == dev) return p;
    SidePool* p = new SidePool;
    p->device = dev;
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    bool ok = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming) == cudaSuccess &&
              cudaStreamCreateWithPriority(&p->hi, cudaStreamNonBlocking, greatest) == cudaSuccess;
    for (int i = 0; i < 3 && ok; ++i) ok = cudaEventCreateWithFlags(&p->gate[i], cudaEventDisableTiming) == cudaSuccess;
    for (int i = 0; i <= kTimelinePoints && ok; ++i) ok = cudaEventCreate(&p->tl[i]) == cudaSuccess;
    for (int i = 0; i < 32 && ok; ++i) ok = cudaEventCreateWithFlags(&p->chunk[i], cudaEventDisableTiming) == cudaSuccess;
    for (int i = 0; i < 10 && ok; ++i) ok = cudaEventCreateWithFlags(&p->blk[i], cudaEventDisableTiming) == cudaSuccess;
    for (int h = 0; h < 2 && ok; ++h) {
        ok = cudaEventCreateWithFlags(&p->wave_gm[h], cudaEventDisableTiming) == cudaSuccess;
        for (int i = 0; i < kWaveStreams && ok; ++i)
            ok = cudaEventCreateWithFlags(&p->wave_pk[h][i], cudaEventDisableTiming) == cudaSuccess &&
                 cudaEventCreateWithFlags(&p->wave_sc[h][i], cudaEventDisableTiming) == cudaSuccess;
    }
    for (int i = 0; i < kSideStreams && ok; ++i)
        ok = cudaStreamCreateWithFlags(&p->s[i], cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&p->join[i], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        return nullptr;   /* the batch then runs on the caller's stream alone */
    }
    g_side.push_back(p);
    return p;
}

int side_fork(SidePool* p, cudaStream_t st)
{
    if (!p) return FMM_OK;
    if (cudaEventRecord(p->fork, st) != cudaSuccess) return FMM_ERR_CUDA;
    for (int i = 0; i < kSideStreams; ++i)
        if (cudaStreamWaitEvent(p->s[i], p->fork, 0) != cudaSuccess) return FMM_ERR_CUDA;
    return FMM_OK;
}

int side_join(SidePool* p, cudaStream_t st)
{
    if (!p) return FMM_OK;
    for (int i = 0; i < kSideStreams; ++i)
        if (cudaEventRecord(p->join[i], p->s[i]) != cudaSuccess || cudaStreamWaitEvent(st, p->join[i], 0) != cudaSuccess)
            return FMM_ERR_CUDA;
    return FMM_OK;
}

/* one side stream (s[0]) beside the caller's stream */
int side_fork1(SidePool* p, cudaStream_t st)
{
    if (cudaEventRecord(p->fork, st) != cudaSuccess) return FMM_ERR_CUDA;
    return cudaStreamWaitEvent(p->s[0], p->fork, 0) == cudaSuccess ? FMM_OK : FMM_ERR_CUDA;
}

int side_join1(SidePool* p, cudaStream_t st)
{
    if (cudaEventRecord(p->join[0], p->s[0]) != cudaSuccess) return FMM_ERR_CUDA;
    return cudaStreamWaitEvent(st, p->join[0], 0) == cudaSuccess ? FMM_OK : FMM_ERR_CUDA;
}

/* per-sub-block row maxima of A (amax) */
static int job_maxima_a(SplitJob& j, cudaStream_t st)
{
    unsigned long long* amax = (unsigned long long*)(j.w + j.L.amax);
    if (cudaMemsetAsync(amax, 0, sizeof(unsigned long long) * (size_t)j.alg.kt * (size_t)j.m, st) != cudaSuccess)
        return FMM_ERR_CUDA;
    /* columns per block: 256, halved (down to 32) while the grid has fewer
     * than 8 blocks per SM, so short-and-wide A still fills the GPU */
    const int64_t rows_blocks = (j.m + 255) / 256 * j.alg.kt;
    int cpb = 256;
    while (cpb > 32 && rows_blocks * ((j.d.ke + cpb - 1) / cpb) < 8 * 152) cpb /= 2;
    dim3 grid((unsigned)((j.m + 255) / 256), (unsigned)j.alg.kt, (unsigned)((j.d.ke + cpb - 1) / cpb));
    amax_kernel<<<grid, 256, 0, st>>>(j.A, j.lda, j.m, j.k, j.alg.kt, amax, cpb, 0, j.m);
    fmm_count_launch(1);
    return FMM_OK;
}

/* per-sub-block column maxima of B (bmax) for the B columns [c0, c1) */
static void job_maxima_b(SplitJob& j, cudaStream_t st, int64_t c0 = 0, int64_t c1 = -1)
{
    if (c1 < 0) c1 = j.n;
    if (c1 <= c0) return;
    unsigned long long* bmax = (unsigned long long*)(j.w + j.L.bmax);
    const int64_t warps = (c1 - c0) * j.alg.kt;
    bmax_kernel<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, st>>>(j.B, j.ldb, j.k, j.n, j.alg.kt, bmax, c0,
                                                                      c1);
    fmm_count_launch(1);
}

/* C := beta*C and the per-sub-block row/column maxima of A and B; with a
 * side pool the B maxima run on its stream s[0], which job_pack joins back */
static int job_prologue(SplitJob& j, cudaStream_t st, SidePool* sp = nullptr)
{
    int rc = fmm_scale_c(j.m, j.n, j.beta, j.C, j.ldc, st);
    if (rc != FMM_OK || j.trivial) return rc;
    if ((rc = job_maxima_a(j, st)) != FMM_OK) return rc;
    if (sp && (rc = side_fork1(sp, st)) != FMM_OK) return rc;
    job_maxima_b(j, sp ? sp->s[0] : st);
    return FMM_OK;
}

/* exponents and digit slices of products [r0, r0 + np); np never exceeds
 * the group the job's workspace was laid out for */
static int job_pack(SplitJob& j, int r0, int np, cudaStream_t st, SidePool* sp = nullptr, bool small = false)
{
    if (np > j.L.group) return FMM_ERR_WORKSPACE;
    const Dims& d = j.d;
    unsigned long long* amax = (unsigned long long*)(j.w + j.L.amax);
    unsigned long long* bmax = (unsigned long long*)(j.w + j.L.bmax);
    int* e_row = (int*)(j.w + j.L.erow);
    int* f_col = (int*)(j.w + j.L.fcol);
    uint8_t* sa = j.w + j.L.sa;
    uint8_t* sb = j.w + j.L.sb;
    if (np <= 0) return FMM_OK;
    /* one launch per kernel for the whole group (grid y holds the product of
     * the exponent pass; the pack grids' x extent np * tiles stays far below
     * 2^31 since np * s * max(m_pad, n_pad) < 2^31) */
    /* A side (row exponents, A slices) on st; B side (column exponents, B
     * slices) on the side stream, after the B maxima queued there */
    cudaStream_t stb = sp ? sp->s[0] : st;
    exps_kernel<<<dim3((unsigned)((d.m_pad + 255) / 256), (unsigned)np), 256, 0, st>>>(
        j.alg.tab, r0, j.m, j.n, j.k, d.m_pad, d.n_pad, amax, bmax, e_row, f_col, 0, d.m_pad);
    int rc;
    if (sp && (rc = side_fork1(sp, st)) != FMM_OK) return rc;
    exps_kernel<<<dim3((unsigned)((d.n_pad + 255) / 256), (unsigned)np), 256, 0, stb>>>(
        j.alg.tab, r0, j.m, j.n, j.k, d.m_pad, d.n_pad, amax, bmax, e_row, f_col, d.m_pad, d.m_pad + d.n_pad);
    PackSel sel;
    sel.small = small;
    launch_packs(j.fmt, j.s, j.alg.tab, r0, np, j.A, j.lda, j.B, j.ldb, j.m, j.n, j.k, d.m_pad, d.n_pad, d.k_pad, e_row,
                 f_col, sa, sb, st, stb, sel);
    if (sp && (rc = side_join1(sp, st)) != FMM_OK) return rc;
    fmm_count_launch(4);
    return FMM_OK;
}

/* The two sides of job_pack separately, for a caller that receives B in
 * column chunks: the A side (row exponents, A slices) and the B side over
 * the T_r columns [j0, j1) (multiples of 32, or j1 = n_pad). */
static void job_pack_a(SplitJob& j, int r0, int np, cudaStream_t st)
{
    const Dims& d = j.d;
    exps_kernel<<<dim3((unsigned)((d.m_pad + 255) / 256), (unsigned)np), 256, 0, st>>>(
        j.alg.tab, r0, j.m, j.n, j.k, d.m_pad, d.n_pad, (unsigned long long*)(j.w + j.L.amax),
        (unsigned long long*)(j.w + j.L.bmax), (int*)(j.w + j.L.erow), (int*)(j.w + j.L.fcol), 0, d.m_pad);
    PackSel sel;
    sel.b = false;
    launch_packs(j.fmt, j.s, j.alg.tab, r0, np, j.A, j.lda, j.B, j.ldb, j.m, j.n, j.k, d.m_pad, d.n_pad, d.k_pad,
                 (int*)(j.w + j.L.erow), (int*)(j.w + j.L.fcol), j.w + j.L.sa, j.w + j.L.sb, st, st, sel);
    fmm_count_launch(2);
}

/* small: the 128-thread pack tiles, which fit on an SM beside a resident
 * GEMM CTA */
static void job_pack_b_cols(SplitJob& j, int r0, int np, int64_t j0, int64_t j1, cudaStream_t st,
                            bool small = false)
{
    const Dims& d = j.d;
    if (j1 <= j0) return;
    exps_kernel<<<dim3((unsigned)((j1 - j0 + 255) / 256), (unsigned)np), 256, 0, st>>>(
        j.alg.tab, r0, j.m, j.n, j.k, d.m_pad, d.n_pad, (unsigned long long*)(j.w + j.L.amax),
        (unsigned long long*)(j.w + j.L.bmax), (int*)(j.w + j.L.erow), (int*)(j.w + j.L.fcol), d.m_pad + j0,
        d.m_pad + j1);
    PackSel sel;
    sel.a = false;
    sel.jb0 = j0;
    sel.jb1 = j1;
    sel.small = small;
    launch_packs(j.fmt, j.s, j.alg.tab, r0, np, j.A, j.lda, j.B, j.ldb, j.m, j.n, j.k, d.m_pad, d.n_pad, d.k_pad,
                 (int*)(j.w + j.L.erow), (int*)(j.w + j.L.fcol), j.w + j.L.sa, j.w + j.L.sb, st, st, sel);
    fmm_count_launch(2);
}

/* per-sub-block row maxima of A (amax, zeroed beforehand) for the
 * product-grid rows [a, b): the A rows ro_p + [a, b) of every row part p */
static void job_maxima_a_rows(SplitJob& j, cudaStream_t st, int64_t a, int64_t b)
{
    unsigned long long* amax = (unsigned long long*)(j.w + j.L.amax);
    for (int p = 0; p < j.alg.mt; ++p) {
        int64_t ro, rl;
        fmm_part_geom(j.m, j.alg.mt, p, &ro, &rl);
        const int64_t r0 = ro + std::min(a, rl), r1 = ro + std::min(b, rl);
        if (r1 <= r0) continue;
        const int64_t rows_blocks = (r1 - r0 + 255) / 256 * j.alg.kt;
        int cpb = 256;
        while (cpb > 32 && rows_blocks * ((j.d.ke + cpb - 1) / cpb) < 8 * 152) cpb /= 2;
        dim3 grid((unsigned)((r1 - r0 + 255) / 256), (unsigned)j.alg.kt, (unsigned)((j.d.ke + cpb - 1) / cpb));
        amax_kernel<<<grid, 256, 0, st>>>(j.A, j.lda, j.m, j.k, j.alg.kt, amax, cpb, r0, r1);
        fmm_count_launch(1);
    }
}

/* row exponents and A slices of the products r0 .. r0+np-1 for the S_r rows
 * [a, b) (multiples of 64, or b = m_pad) */
static void job_pack_a_rows(SplitJob& j, int r0, int np, int64_t a, int64_t b, cudaStream_t st, bool small = false)
{
    const Dims& d = j.d;
    if (b <= a) return;
    exps_kernel<<<dim3((unsigned)((b - a + 255) / 256), (unsigned)np), 256, 0, st>>>(
        j.alg.tab, r0, j.m, j.n, j.k, d.m_pad, d.n_pad, (unsigned long long*)(j.w + j.L.amax),
        (unsigned long long*)(j.w + j.L.bmax), (int*)(j.w + j.L.erow), (int*)(j.w + j.L.fcol), a, b);
    PackSel sel;
    sel.b = false;
    sel.ia0 = a;
    sel.ia1 = b;
    sel.small = small;
    launch_packs(j.fmt, j.s, j.alg.tab, r0, np, j.A, j.lda, j.B, j.ldb, j.m, j.n, j.k, d.m_pad, d.n_pad, d.k_pad,
                 (int*)(j.w + j.L.erow), (int*)(j.w + j.L.fcol), j.w + j.L.sa, j.w + j.L.sb, st, st, sel);
    fmm_count_launch(2);
}

/* G, the level whose unit Z counts in: BF16 6, or 7 when k_pad <= 128 (the
 * finest unit keeping Z inside int64); FP8 s + 1 up to 10 (exact for s <= 9) */
static int job_zlevel(const SplitJob& j)
{
    if (j.fmt) return std::min(j.s + 1, 10);
    return j.d.k_pad <= 128 ? 7 : 6;
}
static int job_db(const SplitJob& j) { return j.fmt ? 5 : 8; }
/* exponent of Z's unit relative to 2^(E_i + F_j) */
static int job_ebase(const SplitJob& j) { return 2 - job_db(j) * job_zlevel(j); }

/* the job's product group as one problem of a GEMM launch */
/* pair tiles for this job's single-call GEMM launches */
static bool job_pair(const SplitJob& j)
{
    return j.d.me >= g_pair_rows.load(std::memory_order_relaxed) && j.d.m_pad % kPairTileM == 0;
}

/* products [r_first, r_first + np) of the job's group as one problem of a
 * GEMM launch: the tensor maps and Z start at product r_first */
static int job_fill(const SplitJob& j, GemmProblem& gp, int np, int item_begin, bool pair = false, int r_first = 0)
{
    const Dims& d = j.d;
    const size_t esz = j.fmt ? 1 : 2;
    const uint8_t* sa = j.w + j.L.sa + (size_t)r_first * j.s * d.m_pad * d.k_pad * esz;
    const uint8_t* sb = j.w + j.L.sb + (size_t)r_first * j.s * d.n_pad * d.k_pad * esz;
    if (make_slice_map(&gp.tmA, sa, d.k_pad, (int64_t)np * j.s * d.m_pad, kTileM, j.fmt) != FMM_OK)
        return FMM_ERR_CUDA;
    if (make_slice_map(&gp.tmB, sb, d.k_pad, (int64_t)np * j.s * d.n_pad, pair ? kTileN / 2 : kTileN, j.fmt) != FMM_OK)
        return FMM_ERR_CUDA;
    gp.Z = (int64_t*)(j.w + j.L.z) + (size_t)r_first * d.m_pad * d.n_pad;
    gp.s = j.s;
    gp.zlevel = job_zlevel(j);
    gp.kbe = kbe_of(j.fmt);
    gp.nkb = (int)(d.k_pad / gp.kbe);
    gp.db = job_db(j);
    gp.fmt = j.fmt;
    gp.m_pad = (int)d.m_pad;
    gp.n_pad = (int)d.n_pad;
    gp.tiles_m = (int)(d.m_pad / (pair ? kPairTileM : kTileM));
    gp.tiles_n = (int)(d.n_pad / kTileN);
    gp.item_begin = item_begin;
    return FMM_OK;
}

static int64_t job_items(const SplitJob& j, int np, bool pair = false)
{
    return (int64_t)np * (j.d.m_pad / (pair ? kPairTileM : kTileM)) * (j.d.n_pad / kTileN);
}

static int launch_gemm(GemmLaunch& gl, int64_t nitems, int nprod_timed, cudaStream_t st, bool pair);

/* The GEMM of the job's current product group, as back-to-back launches of
 * at most K products, K the fewest products that give each launch about 24
 * rounds of work items over the GPU. When the kernels took their items round
 * robin, the persistent CTAs drifted apart over a long launch and shared
 * fewer operand panels in L2, and a new launch started them together again
 * (measured at 16384, two Strassen levels: 92-96 ms of GEMM per step in one
 * launch of 49 products, 86-87 ms in launches of 7). With items drawn
 * dynamically the pair kernel measured the same with 2 or 7 launches per
 * step. */
static int job_gemm(const SplitJob& j, int np, cudaStream_t st)
{
    const bool pair = job_pair(j);
    const int64_t tiles = job_items(j, 1, pair);
    const int64_t units = pair ? 76 : 152;
    int K = (int)std::min<int64_t>(np, std::max<int64_t>(1, (24 * units + tiles - 1) / tiles));
    const int nl = (np + K - 1) / K;
    K = (np + nl - 1) / nl;
    GemmLaunch gl;
    for (int r = 0; r < np; r += K) {
        const int cnt = std::min(K, np - r);
        memset(&gl, 0, sizeof(gl));
        gl.nprob = 1;
        gl.sched = (unsigned int*)(j.w + j.L.sched);
        if (int rc = job_fill(j, gl.prob[0], cnt, 0, pair, r); rc != FMM_OK) return rc;
        if (int rc = launch_gemm(gl, job_items(j, cnt, pair), cnt, st, pair); rc != FMM_OK) return rc;
    }
    return FMM_OK;
}

/* job_gemm restricted to the tile rows [it0, it1) and tile columns
 * [jt0, jt1) of every product: the A slice map starts it0 tile rows
 * further, the B slice map jt0 * 256 rows further and Z at (it0 tile rows,
 * jt0 * 256 columns), with the same row strides, so each (product, tile)
 * item computes exactly what the full launch computes for it. */
static int job_gemm_block(const SplitJob& j, int np, int64_t it0, int64_t it1, int64_t jt0, int64_t jt1,
                          cudaStream_t st)
{
    const bool pair = job_pair(j);
    const int64_t tm = it1 - it0, tn = jt1 - jt0;
    if (tm <= 0 || tn <= 0) return FMM_OK;
    const int64_t tiles = tm * tn;
    const int64_t units = pair ? 76 : 152;
    int K = (int)std::min<int64_t>(np, std::max<int64_t>(1, (24 * units + tiles - 1) / tiles));
    const int nl = (np + K - 1) / K;
    K = (np + nl - 1) / nl;
    const size_t esz = j.fmt ? 1 : 2;
    const int64_t r0 = it0 * (pair ? kPairTileM : kTileM), c0 = jt0 * kTileN;
    GemmLaunch gl;
    for (int r = 0; r < np; r += K) {
        const int cnt = std::min(K, np - r);
        memset(&gl, 0, sizeof(gl));
        gl.nprob = 1;
        gl.sched = (unsigned int*)(j.w + j.L.sched);
        GemmProblem& gp = gl.prob[0];
        if (int rc = job_fill(j, gp, cnt, 0, pair, r); rc != FMM_OK) return rc;
        const uint8_t* sa = j.w + j.L.sa + ((size_t)r * j.s * j.d.m_pad + (size_t)r0) * j.d.k_pad * esz;
        const uint8_t* sb = j.w + j.L.sb + ((size_t)r * j.s * j.d.n_pad + (size_t)c0) * j.d.k_pad * esz;
        if (make_slice_map(&gp.tmA, sa, j.d.k_pad, (int64_t)cnt * j.s * j.d.m_pad - r0, kTileM, j.fmt) != FMM_OK ||
            make_slice_map(&gp.tmB, sb, j.d.k_pad, (int64_t)cnt * j.s * j.d.n_pad - c0, pair ? kTileN / 2 : kTileN,
                           j.fmt) != FMM_OK)
            return FMM_ERR_CUDA;
        gp.Z += r0 + c0 * j.d.m_pad;
        gp.tiles_m = (int)tm;
        gp.tiles_n = (int)tn;
        if (int rc = launch_gemm(gl, (int64_t)cnt * tiles, cnt, st, pair); rc != FMM_OK) return rc;
    }
    return FMM_OK;
}

/* blocks of the grid-stride element-major scatter: one per T elements, at
 * most 16 per SM (each then serves several elements) */
static unsigned scatter_blocks(uint64_t elems, int T)
{
    return (unsigned)std::min<uint64_t>((elems + T - 1) / T, 16 * 152);
}

/* the element-major scatter applies to this job (see job_scatter) */
static bool job_scatter_all(const SplitJob& j, int r0, int np, int* T_out, size_t* smem_out)
{
    const Tab ht = tab_view(j.alg.htab);
    const int P = j.alg.mt * j.alg.nt;
    const int E = ht.w_off[r0 + np] - ht.w_off[r0];
    const int T = std::min(256, kScatterAllSmem / (8 * P)) / 32 * 32;
    const size_t smem = (size_t)P * std::max(T, 0) * 8 + (size_t)E * 12 + (size_t)(np + 1) * 4;
    *T_out = T;
    *smem_out = smem;
    return P <= 64 && T >= 32 && smem <= 47 * 1024;
}

/* the C updates of products [r0, r0 + np) for the product-grid rows
 * [i0, i1) of the columns [j0, j1), element-major form only */
static void job_scatter_block(const SplitJob& j, int r0, int np, int64_t i0, int64_t i1, int64_t j0, int64_t j1,
                              cudaStream_t st, bool small = false)
{
    int T;
    size_t smem;
    job_scatter_all(j, r0, np, &T, &smem);
    if (small && T > 128) {   /* 128-thread blocks fit on an SM beside a resident GEMM CTA */
        const Tab ht = tab_view(j.alg.htab);
        const int P = j.alg.mt * j.alg.nt, E = ht.w_off[r0 + np] - ht.w_off[r0];
        T = 128;
        smem = (size_t)P * T * 8 + (size_t)E * 12 + (size_t)(np + 1) * 4;
    }
    const uint64_t rows = (uint64_t)(i1 - i0);
    const uint64_t first = (uint64_t)j0 * rows, end = (uint64_t)j1 * rows;
    if (end <= first) return;
    scatter_all_kernel<<<scatter_blocks(end - first, T), (unsigned)T, smem, st>>>(
        j.alg.tab, r0, np, j.m, j.n, (int)j.d.m_pad, (int)j.d.n_pad, job_ebase(j), j.alpha,
        (const int64_t*)(j.w + j.L.z), (const int*)(j.w + j.L.erow), (const int*)(j.w + j.L.fcol), j.C, j.ldc, first,
        end, (uint32_t)i0, (uint32_t)rows);
    fmm_count_launch(1);
}

/* the C updates of products [r0, r0 + np) for the product-grid columns
 * [j0, j1) (all rows), element-major form only */
static void job_scatter_cols(const SplitJob& j, int r0, int np, int64_t j0, int64_t j1, cudaStream_t st,
                             bool small = false)
{
    job_scatter_block(j, r0, np, 0, j.d.me, j0, j1, st, small);
}

/* small: blocks of at most 128 threads (and so at most 16 KB of sub-block
 * values), which fit on an SM beside a resident GEMM CTA */
static void job_scatter(const SplitJob& j, int r0, int np, cudaStream_t st, bool small = false)
{
    const int64_t elems = j.d.me * j.d.ne;   /* the largest part's extent */
    /* element-major form when the sub-block values and the group's W entries
     * fit beside the kernel's 1 KB of static geometry in 48 KB: threads per
     * block T = 32 KB / (8 P), a multiple of 32, at least 32 */
    const Tab ht = tab_view(j.alg.htab);
    const int P = j.alg.mt * j.alg.nt;
    const int E = ht.w_off[r0 + np] - ht.w_off[r0];
    int T = std::min(small ? 128 : 256, kScatterAllSmem / (8 * P)) / 32 * 32;
    const size_t smem = (size_t)P * std::max(T, 0) * 8 + (size_t)E * 12 + (size_t)(np + 1) * 4;
    if (P <= 64 && T >= 32 && smem <= 47 * 1024) {
        scatter_all_kernel<<<scatter_blocks((uint64_t)elems, T), (unsigned)T, smem, st>>>(
            j.alg.tab, r0, np, j.m, j.n, (int)j.d.m_pad, (int)j.d.n_pad, job_ebase(j), j.alpha,
            (const int64_t*)(j.w + j.L.z), (const int*)(j.w + j.L.erow), (const int*)(j.w + j.L.fcol), j.C, j.ldc,
            (uint64_t)0, (uint64_t)elems, 0u, 0u);
        fmm_count_launch(1);
        return;
    }
    scatter_kernel<<<dim3((unsigned)((elems + 255) / 256), (unsigned)(j.alg.mt * j.alg.nt)), 256, 0, st>>>(
        j.alg.tab, r0, np, j.m, j.n, (int)j.d.m_pad, (int)j.d.n_pad, job_ebase(j), j.alpha,
        (const int64_t*)(j.w + j.L.z), (const int*)(j.w + j.L.erow), (const int*)(j.w + j.L.fcol), j.C, j.ldc);
    fmm_count_launch(1);
}

static int launch_gemm(GemmLaunch& gl, int64_t nitems, int nprod_timed, cudaStream_t st, bool pair)
{
    /* the kernels' shared-memory limit is a per-device attribute: set once per device */
    static std::atomic<uint64_t> attr_set{0};
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) != cudaSuccess) return FMM_ERR_CUDA;
    const uint64_t bit = dev < 64 ? 1ull << dev : 0;
    if (bit == 0 || !(attr_set.load(std::memory_order_acquire) & bit)) {
        if (cudaFuncSetAttribute(split_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kGemmSmem) != cudaSuccess ||
            cudaFuncSetAttribute(split_gemm_pair_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kPairSmem) != cudaSuccess)
            return FMM_ERR_CUDA;
        attr_set.fetch_or(bit, std::memory_order_acq_rel);
    }
    if (nitems > 0x7fffffffLL) return FMM_ERR_UNSUPPORTED;
    if (nitems == 0) return FMM_OK;
    gl.nitems = (int)nitems;
    gl.err = fmm_device_error_word();
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const bool timed = g_timing;
    if (timed) {
        timing_mark(st, true);
        std::lock_guard<std::mutex> lk(g_timing_mu);
        g_timed_products += (uint64_t)nprod_timed;
    }
    /* both kernels draw their work items from gl.sched, zero at launch */
    if (gl.sched == nullptr || cudaMemsetAsync(gl.sched, 0, sizeof(unsigned int), st) != cudaSuccess)
        return FMM_ERR_CUDA;
    if (pair)   /* clusters of two CTAs, one pair tile each at a time */
        split_gemm_pair_kernel<<<(unsigned)(2 * std::min<int64_t>(nitems, sms / 2)), kGemmThreads, kPairSmem, st>>>(gl);
    else
        split_gemm_kernel<<<(unsigned)std::min<int64_t>(nitems, sms), kGemmThreads, kGemmSmem, st>>>(gl);
    if (timed) timing_mark(st, false);
    fmm_count_launch(1);
    return FMM_OK;
}

/* Two product groups whose work overlaps: the products split into
 * G1 = ceil(R/2) and R - G1, each group with its own exponents, slices and
 * Z (the second region follows the first; the maxima are shared). Group 1
 * is packed with the whole GPU; group 2's packs (small tiles, pool stream
 * s[3]) then run on the SMs beside group 1's GEMM, and group 1's C updates
 * (small blocks, s[4]) beside group 2's GEMM; group 2's C updates follow on
 * s[4], so every C element still receives the products in increasing order
 * and the result is the single group's bit for bit. The second region's
 * layout: the group part of L1 shifted by its own size. */
struct OverlapPlan {
    WsLayout L1;
    size_t shift = 0;
    bool ok = false;
};

static OverlapPlan overlap_plan(const AlgView& alg, const Dims& d, int64_t m, int64_t n, int s, int fmt,
                                size_t bytes)
{
    OverlapPlan o;
    if (alg.R < 2) return o;
    const int G1 = (alg.R + 1) / 2;
    o.L1 = ws_layout_g(alg, d, m, n, s, G1, fmt);
    o.shift = o.L1.total - o.L1.erow;
    /* each group's GEMM keeps every SM busy for at least 8 rounds of items */
    const int64_t tiles = (d.m_pad / (d.me >= kPairMinRows ? kPairTileM : kTileM)) * (d.n_pad / kTileN);
    o.ok = o.L1.total + o.shift <= bytes && (int64_t)G1 * tiles >= 8 * 152 &&
           (int64_t)G1 * s * std::max(d.m_pad, d.n_pad) <= 0x7fffffffLL;
    return o;
}

static int split_overlap(SplitJob& j, const OverlapPlan& o, void* ws, cudaStream_t st, SidePool* sp)
{
    const int R = j.alg.R, G1 = o.L1.group, G2 = R - G1;
    j.L = o.L1;
    j.w = (uint8_t*)ws;
    SplitJob j2 = j;
    j2.L.erow += o.shift;
    j2.L.fcol += o.shift;
    j2.L.sa += o.shift;
    j2.L.sb += o.shift;
    j2.L.z += o.shift;
    j2.L.total += o.shift;
    /* the GEMMs on the greatest-priority stream, so the block scheduler
     * places their CTAs first and the side work fills the room they leave */
    cudaStream_t sg = sp->hi, sp2 = sp->s[3], ssc = sp->s[4];
    auto ok = [](cudaError_t e) { return e == cudaSuccess; };
    int rc;
    if ((rc = job_prologue(j, st, sp)) != FMM_OK) return rc;
    if ((rc = job_pack(j, 0, G1, st, sp)) != FMM_OK) return rc;
    if (!ok(cudaEventRecord(sp->chunk[0], st)) || !ok(cudaStreamWaitEvent(sg, sp->chunk[0], 0))) return FMM_ERR_CUDA;
    if ((rc = job_gemm(j, G1, sg)) != FMM_OK) return rc;
    if (!ok(cudaEventRecord(sp->chunk[2], sg))) return FMM_ERR_CUDA;
    /* group 2's packs after the maxima (and group 1's packs), beside GEMM 1 */
    if (!ok(cudaStreamWaitEvent(sp2, sp->chunk[0], 0))) return FMM_ERR_CUDA;
    if ((rc = job_pack(j2, G1, G2, sp2, nullptr, true)) != FMM_OK) return rc;
    if (!ok(cudaEventRecord(sp->chunk[1], sp2))) return FMM_ERR_CUDA;
    /* group 1's C updates beside GEMM 2 */
    if (!ok(cudaStreamWaitEvent(ssc, sp->chunk[2], 0))) return FMM_ERR_CUDA;
    job_scatter(j, 0, G1, ssc, true);
    if (!ok(cudaStreamWaitEvent(sg, sp->chunk[1], 0))) return FMM_ERR_CUDA;
    if ((rc = job_gemm(j2, G2, sg)) != FMM_OK) return rc;
    if (!ok(cudaEventRecord(sp->chunk[3], sg)) || !ok(cudaStreamWaitEvent(ssc, sp->chunk[3], 0))) return FMM_ERR_CUDA;
    job_scatter(j2, G1, G2, ssc);
    if (!ok(cudaEventRecord(sp->chunk[4], ssc)) || !ok(cudaStreamWaitEvent(st, sp->chunk[4], 0))) return FMM_ERR_CUDA;
    return cudaGetLastError() == cudaSuccess ? FMM_OK : FMM_ERR_CUDA;
}

static int split_launch_budget(const AlgView& alg, int64_t m, int64_t n, int64_t k, double alpha,
                               const double* A, int64_t lda, const double* B, int64_t ldb, double beta,
                               double* C, int64_t ldc, int s, int fmt, void* ws, size_t ws_bytes, size_t budget,
                               cudaStream_t st, SidePool* sp)
{
    SplitJob j;
    int rc = job_init(j, alg, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, s, fmt);
    if (rc != FMM_OK) return rc;
    if (!j.trivial && sp && ws != nullptr && ((uintptr_t)ws & 255) == 0) {
        const OverlapPlan o = overlap_plan(alg, j.d, m, n, s, fmt, std::min(ws_bytes, budget));
        if (o.ok) return split_overlap(j, o, ws, st, sp);
    }
    if (!j.trivial && (rc = job_bind(j, ws, ws_bytes, budget)) != FMM_OK) return rc;
    if ((rc = job_prologue(j, st, sp)) != FMM_OK || j.trivial) return rc;
    const int G = j.L.group;
    for (int r0 = 0; r0 < alg.R; r0 += G) {
        const int np = std::min(G, alg.R - r0);
        if ((rc = job_pack(j, r0, np, st, sp)) != FMM_OK) return rc;
        if ((rc = job_gemm(j, np, st)) != FMM_OK) return rc;
        job_scatter(j, r0, np, st);
    }
    return cudaGetLastError() == cudaSuccess ? FMM_OK : FMM_ERR_CUDA;
}

/* ---------------------------------------------------------------------------
 * Host-buffer entry.
 *
 * Operands in host memory: the call owns the device copies and overlaps the
 * host<->device traffic with the device work. Copies run on s[1] in the
 * order A, B, C (with the blocked schedule below: A's first row half, B's
 * first column half, A's second half, B's second half, C); the A side (row
 * maxima, row exponents, A slices) starts as soon as its rows have arrived,
 * the B side on s[0] as soon as its columns have, and C is only needed by the
 * C updates, so its upload runs under the GEMM. The host enqueues in the same
 * order, which keeps the overlap when a copy from pageable memory blocks the
 * host until it is staged. Every host copy touches its host pages first
 * (fmm_touch_host). The operand and workspace buffers are kept per device
 * (grow-only) until fmm_gpu_release_host_buffers.
 * ------------------------------------------------------------------------- */
struct HostBuffers {
    uint8_t* p = nullptr;
    size_t bytes = 0;
};
static std::mutex g_hostbuf_mu;
static HostBuffers g_hostbuf[64];

static uint8_t* host_buffers(size_t bytes)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    HostBuffers& h = g_hostbuf[dev];
    if (h.bytes >= bytes) return h.p;
    if (h.p) cudaFree(h.p);
    h.p = nullptr;
    h.bytes = 0;
    if (cudaMalloc(&h.p, bytes) != cudaSuccess) {
        cudaGetLastError();
        h.p = nullptr;
        return nullptr;
    }
    h.bytes = bytes;
    return h.p;
}

static size_t align256(size_t b) { return (b + 255) / 256 * 256; }

constexpr int kChunks = 8;   /* B uploads and C downloads per host-buffer call */

int fmm_split_host(const AlgView& alg, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
                   int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc, int s, int fmt)
{
    if (m == 0 || n == 0) return FMM_OK;
    std::lock_guard<std::mutex> use(g_side_use);
    std::lock_guard<std::mutex> buf(g_hostbuf_mu);
    SidePool* sp = side_pool();
    if (!sp) return FMM_ERR_CUDA;
    cudaStream_t st = sp->s[2], cs = sp->s[1];
    const int64_t ka = std::max<int64_t>(k, 1);
    const bool trivial = k == 0 || alpha == 0.0;
    if (trivial && beta == 1.0) return FMM_OK;
    const size_t bA = trivial ? 0 : align256(sizeof(double) * (size_t)(m * ka));
    const size_t bB = trivial ? 0 : align256(sizeof(double) * (size_t)(ka * n));
    const size_t bC = align256(sizeof(double) * (size_t)(m * n));
    const size_t wsb = trivial ? 0 : align256(fmm_split_ws_bytes(alg, m, n, k, s, fmt));
    uint8_t* base = host_buffers(bA + bB + bC + wsb);
    if (!base) return FMM_ERR_ALLOC;
    double* dA = (double*)base;
    double* dB = (double*)(base + bA);
    double* dC = (double*)(base + bA + bB);
    uint8_t* ws = base + bA + bB + bC;
    const size_t row = sizeof(double) * (size_t)m;
    auto ok = [](cudaError_t e) { return e == cudaSuccess; };
    const bool tline = g_timeline.load() && !trivial;
    const auto host_t0 = std::chrono::steady_clock::now();
    auto mark = [&](int x, cudaStream_t on) { if (tline) cudaEventRecord(sp->tl[x], on); };
    if (trivial) {
        /* C := beta*C */
        if (beta != 0.0 && !ok(fmm_copy2d_async(dC, row, C, sizeof(double) * ldc, row, n, cudaMemcpyHostToDevice, st)))
            return FMM_ERR_CUDA;
        if (int rc = fmm_scale_c(m, n, beta, dC, m, st); rc != FMM_OK) return rc;
    } else {
        SplitJob j;
        int rc = job_init(j, alg, m, n, k, alpha, dA, m, dB, ka, 0.0, dC, m, s, fmt);
        if (rc != FMM_OK) return rc;
        if ((rc = job_bind(j, ws, wsb, wsb)) != FMM_OK) return rc;
        const int G = j.L.group, nt = alg.nt;
        const bool one_group = G >= alg.R;
        cudaStream_t sb = sp->s[0];
        /* Blocked schedule, for one product group with the element-major C
         * update and a product grid of at least two GEMM tiles along a side:
         * the grid splits into up to 2 x 2 blocks of tiles (row halves of A,
         * column halves of B). A's first row half and B's first column half
         * go up first, so the GEMM of block (0, 0) starts after half of each
         * operand; A's second half follows, then B's, and the blocks run in
         * the order (0,0), (1,0), (0,1), (1,1). A block's C elements are final
         * when its GEMM ends: they are updated (beside the next block's GEMM)
         * and read back in four column chunks, so after the last GEMM only
         * the last block's C is left. The work a block's GEMM meets beside
         * it (the other halves' slices, the earlier blocks' C updates) runs
         * in the 128-thread forms that fit on an SM beside a GEMM CTA. Every
         * (product, tile) item and every C element is computed as in the
         * unblocked call: the same bits. */
        {
            const bool pair = job_pair(j);
            const int64_t me = j.d.me, ne = j.d.ne, m_pad = j.d.m_pad, n_pad = j.d.n_pad;
            const int64_t U = pair ? kPairTileM : kTileM;
            const int64_t tiles_m = m_pad / U, tiles_n = n_pad / kTileN;
            const int RH = tiles_m >= 2 ? 2 : 1, CH = tiles_n >= 2 ? 2 : 1;
            int Tchk;
            size_t smchk;
            if (one_group && RH * CH >= 2 && job_scatter_all(j, 0, alg.R, &Tchk, &smchk)) {
                const int mt = alg.mt;
                const int64_t tcm[3] = {0, RH == 2 ? (tiles_m + 1) / 2 : tiles_m, tiles_m};
                const int64_t tcn[3] = {0, CH == 2 ? (tiles_n + 1) / 2 : tiles_n, tiles_n};
                const int64_t rcut[3] = {0, tcm[1] * U, m_pad};          /* S_r row halves */
                const int64_t ccut[3] = {0, tcn[1] * kTileN, n_pad};     /* T_r column halves */
                cudaStream_t ss = sp->s[3], sa = sp->s[4];
                auto up_a = [&](int h) -> int {
                    /* the A rows ro_p + [rcut[h], rcut[h+1]) of every row part p, then that half's A side on s[4] */
                    if (RH == 1) {
                        if (!ok(fmm_copy2d_async(dA, row, A, sizeof(double) * lda, row, k, cudaMemcpyHostToDevice, cs)))
                            return FMM_ERR_CUDA;
                    } else {
                        for (int p = 0; p < mt; ++p) {
                            int64_t ro, rl;
                            fmm_part_geom(m, mt, p, &ro, &rl);
                            const int64_t a = ro + std::min(rcut[h], rl), b = ro + std::min(rcut[h + 1], rl);
                            if (b > a && !ok(fmm_copy2d_async(dA + a, row, A + a, sizeof(double) * lda,
                                                               sizeof(double) * (b - a), k, cudaMemcpyHostToDevice, cs)))
                                return FMM_ERR_CUDA;
                        }
                    }
                    if (!ok(cudaEventRecord(sp->blk[h], cs)) || !ok(cudaStreamWaitEvent(sa, sp->blk[h], 0)))
                        return FMM_ERR_CUDA;
                    if (h == 0 && !ok(cudaMemsetAsync(j.w + j.L.amax, 0,
                                                      sizeof(unsigned long long) * (size_t)alg.kt * (size_t)m, sa)))
                        return FMM_ERR_CUDA;
                    job_maxima_a_rows(j, sa, rcut[h], rcut[h + 1]);
                    job_pack_a_rows(j, 0, alg.R, rcut[h], rcut[h + 1], sa, h == 1);
                    return ok(cudaEventRecord(sp->blk[2 + h], sa)) ? FMM_OK : FMM_ERR_CUDA;
                };
                int xb = 0;
                auto up_b = [&](int h) -> int {
                    /* the T_r columns [ccut[h], ccut[h+1]) in four chunks, each chunk's B side on s[0] */
                    const int64_t w = round_up((ccut[h + 1] - ccut[h] + 3) / 4, 32);
                    for (int64_t j0 = ccut[h]; j0 < ccut[h + 1]; j0 += w, ++xb) {
                        const int64_t j1 = std::min(j0 + w, ccut[h + 1]);
                        for (int c = 0; c < nt; ++c) {
                            int64_t co, cl;
                            fmm_part_geom(n, nt, c, &co, &cl);
                            const int64_t a = co + std::min(j0, cl), b = co + std::min(j1, cl);
                            if (b > a && !ok(fmm_copy2d_async(dB + a * k, sizeof(double) * k, B + a * ldb,
                                                               sizeof(double) * ldb, sizeof(double) * k, b - a,
                                                               cudaMemcpyHostToDevice, cs)))
                                return FMM_ERR_CUDA;
                        }
                        if (!ok(cudaEventRecord(sp->chunk[xb], cs)) || !ok(cudaStreamWaitEvent(sb, sp->chunk[xb], 0)))
                            return FMM_ERR_CUDA;
                        for (int c = 0; c < nt; ++c) {
                            int64_t co, cl;
                            fmm_part_geom(n, nt, c, &co, &cl);
                            job_maxima_b(j, sb, co + std::min(j0, cl), co + std::min(j1, cl));
                        }
                        job_pack_b_cols(j, 0, alg.R, j0, j1, sb, h == 1);
                    }
                    return ok(cudaEventRecord(sp->blk[4 + h], sb)) ? FMM_OK : FMM_ERR_CUDA;
                };
                mark(0, cs);
                if ((rc = up_a(0)) != FMM_OK) return rc;
                if (RH == 1) mark(1, cs);
                if ((rc = up_b(0)) != FMM_OK) return rc;
                if (RH == 2) {
                    if ((rc = up_a(1)) != FMM_OK) return rc;
                    mark(1, cs);
                }
                if (CH == 2 && (rc = up_b(1)) != FMM_OK) return rc;
                mark(2, cs);
                /* C up behind A and B, then C := beta*C, on s[3] */
                if (beta != 0.0 &&
                    (!ok(fmm_copy2d_async(dC, row, C, sizeof(double) * ldc, row, n, cudaMemcpyHostToDevice, cs)) ||
                     !ok(cudaEventRecord(sp->gate[2], cs)) || !ok(cudaStreamWaitEvent(ss, sp->gate[2], 0))))
                    return FMM_ERR_CUDA;
                if ((rc = fmm_scale_c(m, n, beta, dC, m, ss)) != FMM_OK) return rc;
                /* the GEMM blocks on the call's stream */
                const int order[4][2] = {{0, 0}, {1, 0}, {0, 1}, {1, 1}};
                int nq = 0;
                int qr[4], qc[4];
                for (const auto& o : order)
                    if (o[0] < RH && o[1] < CH) {
                        qr[nq] = o[0];
                        qc[nq] = o[1];
                        ++nq;
                    }
                for (int q = 0; q < nq; ++q) {
                    if (!ok(cudaStreamWaitEvent(st, sp->blk[2 + qr[q]], 0)) ||
                        !ok(cudaStreamWaitEvent(st, sp->blk[4 + qc[q]], 0)))
                        return FMM_ERR_CUDA;
                    if (q == 0) mark(3, st);
                    if ((rc = job_gemm_block(j, alg.R, tcm[qr[q]], tcm[qr[q] + 1], tcn[qc[q]], tcn[qc[q] + 1], st)) !=
                        FMM_OK)
                        return rc;
                    if (!ok(cudaEventRecord(sp->blk[6 + q], st))) return FMM_ERR_CUDA;
                }
                mark(4, st);
                /* each block's C updates on s[3] in four column chunks, each
                 * chunk's C elements read back on s[1] */
                int xc = 0;
                for (int q = 0; q < nq; ++q) {
                    if (!ok(cudaStreamWaitEvent(ss, sp->blk[6 + q], 0))) return FMM_ERR_CUDA;
                    const int64_t i0 = rcut[qr[q]], i1 = std::min(rcut[qr[q] + 1], me);
                    const int64_t a0 = ccut[qc[q]], b0 = std::min(ccut[qc[q] + 1], ne);
                    if (i1 <= i0 || b0 <= a0) continue;
                    const int64_t w = std::max<int64_t>((b0 - a0 + 3) / 4, 1);
                    for (int64_t j0 = a0; j0 < b0; j0 += w, ++xc) {
                        const int64_t j1 = std::min(j0 + w, b0);
                        job_scatter_block(j, 0, alg.R, i0, i1, j0, j1, ss, q + 1 < nq);
                        if (!ok(cudaEventRecord(sp->chunk[8 + xc], ss)) ||
                            !ok(cudaStreamWaitEvent(cs, sp->chunk[8 + xc], 0)))
                            return FMM_ERR_CUDA;
                        for (int p = 0; p < mt; ++p) {
                            int64_t ro, rl;
                            fmm_part_geom(m, mt, p, &ro, &rl);
                            const int64_t ra = ro + std::min(i0, rl), rb = ro + std::min(i1, rl);
                            if (rb <= ra) continue;
                            for (int c = 0; c < nt; ++c) {
                                int64_t co, cl;
                                fmm_part_geom(n, nt, c, &co, &cl);
                                const int64_t ca = co + std::min(j0, cl), cb = co + std::min(j1, cl);
                                if (cb > ca &&
                                    !ok(fmm_copy2d_async(C + ra + ca * ldc, sizeof(double) * ldc, dC + ra + ca * m, row,
                                                          sizeof(double) * (rb - ra), cb - ca, cudaMemcpyDeviceToHost,
                                                          cs)))
                                    return FMM_ERR_CUDA;
                            }
                        }
                    }
                }
                mark(5, cs);
                if (!ok(cudaStreamSynchronize(cs)) || !ok(cudaStreamSynchronize(st)) ||
                    !ok(cudaStreamSynchronize(ss)) || !ok(cudaStreamSynchronize(sa)) || !ok(cudaStreamSynchronize(sb)))
                    return FMM_ERR_CUDA;
                if (tline) {
                    std::lock_guard<std::mutex> lk(g_timeline_mu);
                    for (int y = 1; y <= kTimelinePoints; ++y) {
                        float t = 0.f;
                        cudaEventElapsedTime(&t, sp->tl[0], sp->tl[y]);
                        g_timeline_ms[y - 1] = t;
                    }
                    g_timeline_ms[kTimelinePoints] =
                        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - host_t0).count();
                }
                return cudaGetLastError() == cudaSuccess ? fmm_device_error_status() : FMM_ERR_CUDA;
            }
        }
        /* A, then the A side's maxima (and, with one product group, its
         * exponents and slices) */
        mark(0, cs);
        if (!ok(fmm_copy2d_async(dA, row, A, sizeof(double) * lda, row, k, cudaMemcpyHostToDevice, cs)) ||
            !ok(cudaEventRecord(sp->gate[0], cs)) || !ok(cudaStreamWaitEvent(st, sp->gate[0], 0)))
            return FMM_ERR_CUDA;
        mark(1, cs);
        if ((rc = job_maxima_a(j, st)) != FMM_OK) return rc;
        if (one_group) job_pack_a(j, 0, alg.R, st);
        /* B in kChunks chunks of T_r columns [j0, j1): chunk x holds the B
         * columns co_c + [j0, j1) of every column part c, and the B side of
         * those columns (maxima; with one group, exponents and slices) runs
         * on s[0] as soon as the chunk has arrived */
        const int64_t ne = j.d.ne, n_pad = j.d.n_pad;
        const int64_t W = (ne + kChunks * 32 - 1) / (kChunks * 32) * 32;
        int x = 0;
        for (int64_t j0 = 0; j0 < n_pad; j0 += W, ++x) {
            const int64_t j1 = std::min(j0 + W, n_pad);
            for (int c = 0; c < nt; ++c) {
                int64_t co, cl;
                fmm_part_geom(n, nt, c, &co, &cl);
                const int64_t a = co + std::min(j0, cl), b = co + std::min(j1, cl);
                if (b > a && !ok(fmm_copy2d_async(dB + a * k, sizeof(double) * k, B + a * ldb, sizeof(double) * ldb,
                                                   sizeof(double) * k, b - a, cudaMemcpyHostToDevice, cs)))
                    return FMM_ERR_CUDA;
            }
            if (!ok(cudaEventRecord(sp->chunk[x], cs)) || !ok(cudaStreamWaitEvent(sb, sp->chunk[x], 0)))
                return FMM_ERR_CUDA;
            for (int c = 0; c < nt; ++c) {
                int64_t co, cl;
                fmm_part_geom(n, nt, c, &co, &cl);
                job_maxima_b(j, sb, co + std::min(j0, cl), co + std::min(j1, cl));
            }
            if (one_group) job_pack_b_cols(j, 0, alg.R, j0, j1, sb);
        }
        mark(2, cs);
        for (int r0 = 0; r0 < alg.R; r0 += G) {
            const int np = std::min(G, alg.R - r0);
            if (one_group) {
                if ((rc = side_join1(sp, st)) != FMM_OK) return rc;
            } else if ((rc = job_pack(j, r0, np, st, sp)) != FMM_OK) {
                return rc;
            }
            if (r0 == 0) mark(3, st);
            if ((rc = job_gemm(j, np, st)) != FMM_OK) return rc;
            if (r0 + np >= alg.R) mark(4, st);
            if (r0 == 0) {
                /* C under the first GEMM, then C := beta*C before the first scatter */
                if (beta != 0.0 &&
                    (!ok(fmm_copy2d_async(dC, row, C, sizeof(double) * ldc, row, n, cudaMemcpyHostToDevice, cs)) ||
                     !ok(cudaEventRecord(sp->gate[2], cs)) || !ok(cudaStreamWaitEvent(st, sp->gate[2], 0))))
                    return FMM_ERR_CUDA;
                if ((rc = fmm_scale_c(m, n, beta, dC, m, st)) != FMM_OK) return rc;
            }
            int T;
            size_t smem;
            if (r0 + np < alg.R || !job_scatter_all(j, r0, np, &T, &smem)) {
                job_scatter(j, r0, np, st);
                continue;
            }
            /* the last group's C updates in column chunks of the product grid,
             * each chunk's C columns (co_c + [j0, j1) of every column part)
             * read back on s[1] while the next chunk is computed */
            const int64_t W2 = (ne + kChunks - 1) / kChunks;
            x = 0;
            for (int64_t j0 = 0; j0 < ne; j0 += W2, ++x) {
                const int64_t j1 = std::min(j0 + W2, ne);
                job_scatter_cols(j, r0, np, j0, j1, st);
                if (!ok(cudaEventRecord(sp->chunk[kChunks + x], st)) ||
                    !ok(cudaStreamWaitEvent(cs, sp->chunk[kChunks + x], 0)))
                    return FMM_ERR_CUDA;
                for (int c = 0; c < nt; ++c) {
                    int64_t co, cl;
                    fmm_part_geom(n, nt, c, &co, &cl);
                    const int64_t a = co + std::min(j0, cl), b = co + std::min(j1, cl);
                    if (b > a && !ok(fmm_copy2d_async(C + a * ldc, sizeof(double) * ldc, dC + a * m, row, row, b - a,
                                                       cudaMemcpyDeviceToHost, cs)))
                        return FMM_ERR_CUDA;
                }
            }
            mark(5, cs);
            if (!ok(cudaEventRecord(sp->gate[1], cs)) || !ok(cudaStreamSynchronize(cs)) ||
                !ok(cudaStreamSynchronize(st)))
                return FMM_ERR_CUDA;
            if (tline) {
                std::lock_guard<std::mutex> lk(g_timeline_mu);
                for (int x = 1; x <= kTimelinePoints; ++x) {
                    float t = 0.f;
                    cudaEventElapsedTime(&t, sp->tl[0], sp->tl[x]);
                    g_timeline_ms[x - 1] = t;
                }
                g_timeline_ms[kTimelinePoints] =
                    std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - host_t0).count();
            }
            return cudaGetLastError() == cudaSuccess ? fmm_device_error_status() : FMM_ERR_CUDA;
        }
    }
    if (!ok(fmm_copy2d_async(C, sizeof(double) * ldc, dC, row, row, n, cudaMemcpyDeviceToHost, st)) ||
        !ok(cudaStreamSynchronize(st)))
        return FMM_ERR_CUDA;
    /* a kernel whose bounded wait expired left C incomplete: report it */
    return cudaGetLastError() == cudaSuccess ? fmm_device_error_status() : FMM_ERR_CUDA;
}

void fmm_split_host_release()
{
    std::lock_guard<std::mutex> buf(g_hostbuf_mu);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
    if (g_hostbuf[dev].p) cudaFree(g_hostbuf[dev].p);
    g_hostbuf[dev] = HostBuffers();
}

/* Batched split-form GEMMs: problems are taken in order into waves of at
 * most kMaxLaunchProblems whose whole workspaces (all products at once) fit
 * together; per wave every problem is packed, one persistent GEMM launch per
 * tile kind covers all their (problem, product, tile) items, then each
 * problem's C is updated. When the batch needs more than one wave, waves
 * alternate between the two halves of the workspace: a wave's maxima and
 * packs (pack streams s[0..7]) wait only for the C updates of the wave before
 * last, which used the same half, so they run beside the previous wave's GEMM
 * and C updates (scatter streams s[8..15]); the GEMMs run in order on the
 * caller's stream. A problem too large for its share of the workspace runs
 * alone, after everything before it, with the whole workspace and product
 * groups. Every problem's result equals its single-call result. */
/* ------------------------------------------- batched waves: host side ---- */

/* the fields every wave kernel reads, for a bound job (its whole algorithm as one group) */
static WaveProb wave_prob(const SplitJob& j)
{
    WaveProb w;
    memset(&w, 0, sizeof(w));
    w.tab = j.alg.tab;
    w.A = j.A; w.B = j.B; w.C = j.C;
    w.amax = (unsigned long long*)(j.w + j.L.amax);
    w.bmax = (unsigned long long*)(j.w + j.L.bmax);
    w.e_row = (int*)(j.w + j.L.erow);
    w.f_col = (int*)(j.w + j.L.fcol);
    w.sa = j.w + j.L.sa;
    w.sb = j.w + j.L.sb;
    w.Z = (const int64_t*)(j.w + j.L.z);
    w.lda = j.lda; w.ldb = j.ldb; w.ldc = j.ldc;
    w.m = j.m; w.n = j.n; w.k = j.k;
    w.m_pad = j.d.m_pad; w.n_pad = j.d.n_pad; w.k_pad = j.d.k_pad;
    w.alpha = j.alpha; w.beta = j.beta;
    w.R = j.alg.R; w.kt = j.alg.kt;
    w.ebase = job_ebase(j);
    return w;
}

/* a table over jobs `qs`, each given gx and its block count by `size`; returns the launch's blocks */
template <class F>
static int64_t wave_table(WaveLaunch& L, const std::vector<SplitJob*>& qs, F size)
{
    L.nprob = 0;
    int64_t acc = 0;
    for (SplitJob* j : qs) {
        WaveProb& w = L.p[L.nprob++];
        w = wave_prob(*j);
        size(*j, w);
        w.b0 = acc;
        acc += w.nb;
    }
    return acc;
}

template <int S, int DB>
static void wave_packs_t(WaveLaunch& L, const std::vector<SplitJob*>& qs, bool small, cudaStream_t st)
{
    const int rows = small ? 32 : 64, cols = small ? 16 : 32;
    int64_t nb = wave_table(L, qs, [&](const SplitJob& j, WaveProb& w) {
        w.gx = (int64_t)j.alg.R * (j.d.m_pad / rows);
        w.nb = w.gx * (j.d.k_pad / 64);
    });
    if (small)
        wave_pack_a_kernel<S, DB, 32><<<(unsigned)nb, 128, 0, st>>>(L);
    else
        wave_pack_a_kernel<S, DB, 64><<<(unsigned)nb, 256, 0, st>>>(L);
    nb = wave_table(L, qs, [&](const SplitJob& j, WaveProb& w) {
        w.gx = (int64_t)j.alg.R * ((j.d.n_pad + cols - 1) / cols);
        w.nb = w.gx * (j.d.k_pad / 64);
    });
    if (small)
        wave_pack_b_kernel<S, DB, 16><<<(unsigned)nb, 128, 0, st>>>(L);
    else
        wave_pack_b_kernel<S, DB, 32><<<(unsigned)nb, 256, 0, st>>>(L);
    fmm_count_launch(2);
}

static void wave_packs(int fmt, int s, WaveLaunch& L, const std::vector<SplitJob*>& qs, bool small, cudaStream_t st)
{
#define FMM_WPACKS(S_, DB_) wave_packs_t<S_, DB_>(L, qs, small, st)
    if (fmt == 0) {
        switch (s) {
        case 2: FMM_WPACKS(2, 8); break;
        case 3: FMM_WPACKS(3, 8); break;
        case 4: FMM_WPACKS(4, 8); break;
        case 5: FMM_WPACKS(5, 8); break;
        case 6: FMM_WPACKS(6, 8); break;
        case 7: FMM_WPACKS(7, 8); break;
        default: FMM_WPACKS(8, 8); break;
        }
    } else {
        switch (s) {
        case 2: FMM_WPACKS(2, 5); break;
        case 3: FMM_WPACKS(3, 5); break;
        case 4: FMM_WPACKS(4, 5); break;
        case 5: FMM_WPACKS(5, 5); break;
        case 6: FMM_WPACKS(6, 5); break;
        case 7: FMM_WPACKS(7, 5); break;
        case 8: FMM_WPACKS(8, 5); break;
        case 9: FMM_WPACKS(9, 5); break;
        case 10: FMM_WPACKS(10, 5); break;
        case 11: FMM_WPACKS(11, 5); break;
        default: FMM_WPACKS(12, 5); break;
        }
    }
#undef FMM_WPACKS
}

/* The side work before a wave's GEMM, one launch per kernel over the bound
 * jobs qs (all products of each as one group): C scaling and maxima zeroing,
 * maxima, exponents, then the packs per (slice count, format). */
static int wave_side_pack(const std::vector<SplitJob*>& qs, bool small, cudaStream_t st)
{
    if (qs.empty()) return FMM_OK;
    WaveLaunch L;
    int64_t nb = wave_table(L, qs, [](const SplitJob& j, WaveProb& w) {
        const int64_t total = (int64_t)j.alg.kt * (j.m + j.n) + (j.beta != 1.0 ? j.m * j.n : 0);
        w.gx = 1;
        w.nb = std::min<int64_t>(std::max<int64_t>((total + 2047) / 2048, 1), 2048);
    });
    wave_prep_kernel<<<(unsigned)nb, 256, 0, st>>>(L);
    nb = wave_table(L, qs, [](const SplitJob& j, WaveProb& w) {
        w.gx = (j.m + 255) / 256 * j.alg.kt * ((j.d.ke + 255) / 256);
        w.nb = w.gx + ((int64_t)j.alg.kt * j.n * 32 + 255) / 256;
    });
    wave_maxima_kernel<<<(unsigned)nb, 256, 0, st>>>(L);
    nb = wave_table(L, qs, [](const SplitJob& j, WaveProb& w) {
        w.gx = (j.d.m_pad + j.d.n_pad + 255) / 256;
        w.nb = w.gx * j.alg.R;
    });
    wave_exps_kernel<<<(unsigned)nb, 256, 0, st>>>(L);
    fmm_count_launch(3);
    /* packs, one pair of launches per (format, slice count) present */
    std::vector<std::pair<int, int>> kinds;
    for (SplitJob* j : qs)
        if (std::find(kinds.begin(), kinds.end(), std::make_pair(j->fmt, j->s)) == kinds.end())
            kinds.emplace_back(j->fmt, j->s);
    for (auto [fmt, sl] : kinds) {
        std::vector<SplitJob*> sel;
        for (SplitJob* j : qs)
            if (j->fmt == fmt && j->s == sl) sel.push_back(j);
        wave_packs(fmt, sl, L, sel, small, st);
    }
    return cudaGetLastError() == cudaSuccess ? FMM_OK : FMM_ERR_CUDA;
}

/* The C updates after a wave's GEMM: the element-major form in one launch for
 * the jobs whose sub-block values and W entries fit its shared memory, the
 * per-job form for the rest. */
static int wave_side_scatter(const std::vector<SplitJob*>& qs, bool small, cudaStream_t st)
{
    std::vector<SplitJob*> all, other;
    int T = small ? 128 : 256;
    for (SplitJob* j : qs) {
        int Tj;
        size_t sm;
        if (job_scatter_all(*j, 0, j->alg.R, &Tj, &sm) && Tj >= 32) {
            all.push_back(j);
            T = std::min(T, Tj);
        } else {
            other.push_back(j);
        }
    }
    if (!all.empty()) {
        size_t smem = 0;
        for (SplitJob* j : all) {
            const Tab ht = tab_view(j->alg.htab);
            const int P = j->alg.mt * j->alg.nt, E = ht.w_off[j->alg.R] - ht.w_off[0];
            smem = std::max(smem, (size_t)P * T * 8 + (size_t)E * 12 + (size_t)(j->alg.R + 1) * 4);
        }
        WaveLaunch L;
        const int64_t nb = wave_table(L, all, [&](const SplitJob& j, WaveProb& w) {
            w.gx = 1;
            w.nb = scatter_blocks((uint64_t)(j.d.me * j.d.ne), T);
        });
        wave_scatter_kernel<<<(unsigned)nb, (unsigned)T, smem, st>>>(L);
        fmm_count_launch(1);
    }
    for (SplitJob* j : other) job_scatter(*j, 0, j->alg.R, st, small);
    return cudaGetLastError() == cudaSuccess ? FMM_OK : FMM_ERR_CUDA;
}

int fmm_split_batch(int count, const SplitJob* jobs_in, void* ws, size_t ws_bytes, cudaStream_t st)
{
    std::lock_guard<std::mutex> use(g_side_use);
    SidePool* sp = side_pool();
    std::vector<SplitJob> jobs(jobs_in, jobs_in + count);
    std::vector<size_t> full(count, 0);
    size_t total = 0;
    int nontrivial = 0;
    for (int i = 0; i < count; ++i)
        if (!jobs[i].trivial) {
            const WsLayout Lf = ws_layout_g(jobs[i].alg, jobs[i].d, jobs[i].m, jobs[i].n, jobs[i].s, jobs[i].alg.R,
                                            jobs[i].fmt);
            full[i] = Lf.total;
            total += (full[i] + 255) / 256 * 256;
            ++nontrivial;
        }
    /* one wave over the whole workspace when everything fits at once;
     * otherwise two halves that waves alternate between */
    const bool halves = sp != nullptr && (total > ws_bytes || nontrivial > kMaxLaunchProblems);
    const size_t share = halves ? ws_bytes / 2 / 256 * 256 : ws_bytes;
    auto pack_st = [&](int x) { return sp ? sp->s[x % kWaveStreams] : st; };
    auto scat_st = [&](int x) { return sp ? sp->s[kWaveStreams + x % kWaveStreams] : st; };
    auto ok = [](cudaError_t e) { return e == cudaSuccess; };
    bool half_used[2] = {false, false};
    struct Wave {
        int i, e, h;
    };
    int wave = 0;

    /* a wave's maxima, exponents and packs on the pack streams, after the C
     * updates of the last wave in its half; the GEMM stream then waits */
    auto pack_wave = [&](const Wave& W) -> int {
        uint8_t* base = (uint8_t*)ws + (size_t)W.h * share;
        if (sp && half_used[W.h])
            for (int x = 0; x < kWaveStreams; ++x)
                for (int y = 0; y < kWaveStreams; ++y)
                    if (!ok(cudaStreamWaitEvent(pack_st(x), sp->wave_sc[W.h][y], 0))) return FMM_ERR_CUDA;
        size_t off = 0;
        std::vector<SplitJob*> qs;
        for (int q = W.i; q < W.e; ++q) {
            SplitJob& j = jobs[q];
            int rc = job_bind_group(j, base + off, full[q], j.alg.R);
            if (rc != FMM_OK) return rc;
            off += (full[q] + 255) / 256 * 256;
            qs.push_back(&j);
        }
        /* the full-size tiles: measured, a wave's side kernels do not overlap the previous wave's GEMM (its
         * CTAs hold the SMs), so the tiles that fit beside a GEMM CTA only make them slower */
        if (int rc = wave_side_pack(qs, false, pack_st(0)); rc != FMM_OK) return rc;
        if (sp)
            for (int x = 0; x < kWaveStreams; ++x)
                if (!ok(cudaEventRecord(sp->wave_pk[W.h][x], pack_st(x)))) return FMM_ERR_CUDA;
        return FMM_OK;
    };
    /* one persistent GEMM launch per tile kind over the wave's items, the
     * costliest items (slice pairs x k blocks) first so the CTAs' shares end
     * evenly; pair-tile problems and the rest give the same bits per tile */
    auto gemm_wave = [&](const Wave& W) -> int {
        if (sp)
            for (int x = 0; x < kWaveStreams; ++x)
                if (!ok(cudaStreamWaitEvent(st, sp->wave_pk[W.h][x], 0))) return FMM_ERR_CUDA;
        std::vector<int> ord;
        for (int q = W.i; q < W.e; ++q) ord.push_back(q);
        auto item_cost = [&](int q) {
            return (int64_t)jobs[q].s * (jobs[q].s + 1) / 2 * (jobs[q].d.k_pad / kbe_of(jobs[q].fmt)) /
                   (jobs[q].fmt ? 2 : 1);   /* FP8 MMAs run at twice the BF16 rate */
        };
        std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return item_cost(a) > item_cost(b); });
        GemmLaunch gl;
        for (int pass = 0; pass < 2; ++pass) {
            const bool pair = pass == 0;
            memset(&gl, 0, sizeof(gl));
            int64_t items = 0;
            int prods = 0;
            for (int q : ord) {
                SplitJob& j = jobs[q];
                if (job_pair(j) != pair) continue;
                if (gl.sched == nullptr) gl.sched = (unsigned int*)(j.w + j.L.sched);
                int rc = job_fill(j, gl.prob[gl.nprob++], j.alg.R, (int)items, pair);
                if (rc != FMM_OK) return rc;
                items += job_items(j, j.alg.R, pair);
                prods += j.alg.R;
            }
            if (gl.nprob == 0) continue;
            if (int rc = launch_gemm(gl, items, prods, st, pair); rc != FMM_OK) return rc;
        }
        if (sp && !ok(cudaEventRecord(sp->wave_gm[W.h], st))) return FMM_ERR_CUDA;
        return FMM_OK;
    };
    /* each problem's C update (disjoint C regions) on the scatter streams */
    auto scatter_wave = [&](const Wave& W) -> int {
        if (sp)
            for (int y = 0; y < kWaveStreams; ++y)
                if (!ok(cudaStreamWaitEvent(scat_st(y), sp->wave_gm[W.h], 0))) return FMM_ERR_CUDA;
        std::vector<SplitJob*> qs;
        for (int q = W.i; q < W.e; ++q) qs.push_back(&jobs[q]);
        if (int rc = wave_side_scatter(qs, false, scat_st(0)); rc != FMM_OK) return rc;
        if (sp)
            for (int y = 0; y < kWaveStreams; ++y)
                if (!ok(cudaEventRecord(sp->wave_sc[W.h][y], scat_st(y)))) return FMM_ERR_CUDA;
        half_used[W.h] = true;
        return FMM_OK;
    };

    /* software pipeline, enqueued as GEMM(w), packs(w+1), C updates(w): a pack
     * stream that shares a hardware queue with a scatter stream then never
     * has its work behind the C updates' wait for GEMM(w) */
    bool pending = false;
    Wave P{0, 0, 0};
    auto flush = [&]() -> int {
        if (!pending) return FMM_OK;
        pending = false;
        int rc = gemm_wave(P);
        return rc != FMM_OK ? rc : scatter_wave(P);
    };
    if (int rc = side_fork(sp, st); rc != FMM_OK) return rc;   /* side streams start after the caller's work */
    int i = 0;
    while (i < count) {
        if (jobs[i].trivial) {
            int rc = job_prologue(jobs[i], st);
            if (rc != FMM_OK) return rc;
            ++i;
            continue;
        }
        if (full[i] > share) {
            /* alone, after every wave before it, with the whole workspace */
            SplitJob& j = jobs[i];
            int rc = flush();
            if (rc == FMM_OK) rc = side_join(sp, st);
            if (rc == FMM_OK)
                rc = split_launch_budget(j.alg, j.m, j.n, j.k, j.alpha, j.A, j.lda, j.B, j.ldb, j.beta, j.C, j.ldc,
                                         j.s, j.fmt, ws, ws_bytes, ws_bytes, st, sp);
            if (rc == FMM_OK) rc = side_fork(sp, st);
            if (rc != FMM_OK) return rc;
            half_used[0] = half_used[1] = false;
            ++i;
            continue;
        }
        /* gather a wave */
        int e = i;
        size_t used = 0;
        while (e < count && e - i < kMaxLaunchProblems && !jobs[e].trivial && used + full[e] <= share &&
               (int64_t)jobs[e].alg.R * jobs[e].s * std::max(jobs[e].d.m_pad, jobs[e].d.n_pad) <= 0x7fffffffLL) {
            used += (full[e] + 255) / 256 * 256;
            ++e;
        }
        if (e == i) return FMM_ERR_WORKSPACE;
        const Wave W{i, e, halves ? (wave & 1) : 0};
        ++wave;
        int rc = FMM_OK;
        if (halves) {
            /* W packs into the other half than the pending wave */
            if (pending) rc = gemm_wave(P);
            if (rc == FMM_OK) rc = pack_wave(W);
            if (rc == FMM_OK && pending) rc = scatter_wave(P);
        } else {
            /* one region: the pending wave is done with it first */
            rc = flush();
            if (rc == FMM_OK) rc = pack_wave(W);
        }
        if (rc != FMM_OK) return rc;
        P = W;
        pending = true;
        i = e;
    }
    if (int rc = flush(); rc != FMM_OK) return rc;
    if (int rc = side_join(sp, st); rc != FMM_OK) return rc;   /* the caller's stream waits for everything */
    return cudaGetLastError() == cudaSuccess ? FMM_OK : FMM_ERR_CUDA;
}

/* workspace the batch would use with everything in one wave where possible */
size_t fmm_split_batch_ws(int count, const SplitJob* jobs)
{
    size_t sum = 0, mx = 0;
    for (int i = 0; i < count; ++i) {
        if (jobs[i].trivial) continue;
        const size_t f =
            ws_layout_g(jobs[i].alg, jobs[i].d, jobs[i].m, jobs[i].n, jobs[i].s, jobs[i].alg.R, jobs[i].fmt).total;
        sum += (f + 255) / 256 * 256;
        const size_t one = ws_layout(jobs[i].alg, jobs[i].m, jobs[i].n, jobs[i].k, jobs[i].s, 1, jobs[i].fmt).total;
        mx = std::max(mx, one);
    }
    return std::max(std::min(sum, kGroupBudget), mx);
}

int fmm_split_job_make(SplitJob** out, const AlgView& alg, int64_t m, int64_t n, int64_t k, double alpha,
                       const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C,
                       int64_t ldc, int s)
{
    SplitJob* j = new SplitJob;
    int rc = job_init(*j, alg, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, s);
    if (rc != FMM_OK) { delete j; return rc; }
    *out = j;
    return FMM_OK;
}

void fmm_split_job_free(SplitJob* j) { delete j; }

int fmm_split_launch(const AlgView& alg, int64_t m, int64_t n, int64_t k, double alpha,
                     const double* A, int64_t lda, const double* B, int64_t ldb, double beta,
                     double* C, int64_t ldc, int s, int fmt, void* ws, size_t ws_bytes, cudaStream_t st)
{
    /* the group size follows the workspace the caller provides */
    std::lock_guard<std::mutex> use(g_side_use);
    return split_launch_budget(alg, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, s, fmt, ws, ws_bytes,
                               ws_bytes, st, side_pool());
}

/* ---------------------------------------------------------------------------
 * Allocation-free entry point.
 *
 * For callers that must not allocate device memory while they run: stream
 * callbacks and host functions, plug-ins that run on memory handed to them by
 * a host application with its own allocator, or processes whose device memory
 * is already fully reserved. Such callers cannot use fmm_gpu_split_dgemm,
 * whose workspace they would have to obtain, nor the table cache, which
 * allocates on first use of an algorithm. This variant keeps the algorithm
 * table and the whole workspace in one file-scope device array of
 * kNoAllocScratchBytes (64 MiB), which every GPU that loads the library holds
 * until the process exits.
 * ------------------------------------------------------------------------- */
constexpr size_t kNoAllocScratchBytes = (size_t)64 << 20;
static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
std::mutex g_noalloc_mu;
uint8_t* g_noalloc_ptr[64];

/* One piece of an algorithm table, passed by value: the launch copies the
 * values when it is enqueued, so no host buffer has to outlive the call. */
constexpr int kTabChunkInts = 4000;
struct TabChunk {
    int n;
    int v[kTabChunkInts];
};

__global__ void __launch_bounds__(256) noalloc_table_kernel(int* __restrict__ dst, const __grid_constant__ TabChunk c)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < c.n; i += gridDim.x * blockDim.x) dst[i] = c.v[i];
}
}  // namespace

extern "C" int fmm_gpu_split_dgemm_noalloc(const fmm_t* fmm, int levels, int64_t m, int64_t n, int64_t k,
                                           double alpha, const double* A, int64_t lda, const double* B,
                                           int64_t ldb, double beta, double* C, int64_t ldc, int slices,
                                           void* stream)
{
    if (m < 0 || n < 0 || k < 0 || slices < 2 || slices > 8) return FMM_ERR_ARG;
    if (lda < (m > 1 ? m : 1) || ldb < (k > 1 ? k : 1) || ldc < (m > 1 ? m : 1)) return FMM_ERR_ARG;
    if (m > 0 && n > 0 && C == nullptr) return FMM_ERR_ARG;
    if (m > 0 && n > 0 && k > 0 && (A == nullptr || B == nullptr)) return FMM_ERR_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return FMM_ERR_CUDA;
    uint8_t* scratch;
    {
        /* once per device, with that device current: the device address of
         * the static array (its host-side name is only a stand-in) */
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (g_noalloc_ptr[dev] == nullptr) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return FMM_ERR_CUDA;
            g_noalloc_ptr[dev] = (uint8_t*)p;
        }
        scratch = g_noalloc_ptr[dev];
    }
    fmm_t flat;
    int owned = 0;
    int rc = fmm_flatten(fmm, levels, &flat, &owned);
    if (rc != FMM_OK) return rc;
    std::vector<int> table;
    AlgView alg;
    rc = fmm_alg_describe(&flat, &table, &alg);
    if (owned) free_fmm(flat);
    if (rc != FMM_OK) return rc;
    const size_t tab_bytes = (sizeof(int) * table.size() + 255) / 256 * 256;
    if (tab_bytes >= kNoAllocScratchBytes) return FMM_ERR_SCRATCH;
    const size_t ws_bytes = kNoAllocScratchBytes - tab_bytes;
    if (m > 0 && n > 0 && k > 0 && alpha != 0.0 && ws_layout(alg, m, n, k, slices, ws_bytes).total > ws_bytes)
        return FMM_ERR_SCRATCH;
    if (fmm_device_error_word() == nullptr) return FMM_ERR_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    /* the table goes to the front of the scratch, written by kernels that
     * carry it as their parameter (never a copy from this call's host vector,
     * which is gone once the call returns) */
    for (size_t off = 0; off < table.size(); off += kTabChunkInts) {
        TabChunk c;
        c.n = (int)std::min<size_t>(kTabChunkInts, table.size() - off);
        std::memcpy(c.v, table.data() + off, sizeof(int) * (size_t)c.n);
        noalloc_table_kernel<<<(c.n + 255) / 256, 256, 0, st>>>((int*)scratch + off, c);
        if (cudaGetLastError() != cudaSuccess) return FMM_ERR_CUDA;
        fmm_count_launch(1);
    }
    alg.tab = (const int*)scratch;
    alg.htab = table.data();
    return split_launch_budget(alg, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, slices, 0, scratch + tab_bytes,
                               ws_bytes, ws_bytes, st, nullptr);
}

/* ---------------------------------------------------------------------------
 * Batched entry point (include/fmm_gb300.h).
 * ------------------------------------------------------------------------- */
namespace {

/* Validates a batch and describes its problems. With `host_tables` (sizing
 * only) the algorithm tables are built on the host and kept in it, so sizing
 * needs no device; otherwise they are the cached device tables. */
int batch_jobs(int count, const fmm_batch_problem* probs, std::vector<SplitJob>& jobs,
               std::vector<int>& f64_idx, std::vector<AlgView>& f64_alg,
               std::deque<std::vector<int>>* host_tables = nullptr)
{
    if (count < 0 || (count > 0 && probs == nullptr)) return FMM_ERR_ARG;
    for (int i = 0; i < count; ++i) {
        const fmm_batch_problem& p = probs[i];
        if (p.m < 0 || p.n < 0 || p.k < 0) return FMM_ERR_ARG;
        if (p.lda < (p.m > 1 ? p.m : 1) || p.ldb < (p.k > 1 ? p.k : 1) || p.ldc < (p.m > 1 ? p.m : 1))
            return FMM_ERR_ARG;
        if (p.m > 0 && p.n > 0 && p.C == nullptr) return FMM_ERR_ARG;
        if (p.m > 0 && p.n > 0 && p.k > 0 && (p.A == nullptr || p.B == nullptr)) return FMM_ERR_ARG;
        if (p.format != 0 && p.format != 1) return FMM_ERR_ARG;
        if (p.slices != 0 && (p.slices < 2 || p.slices > (p.format ? 12 : 8))) return FMM_ERR_ARG;
        fmm_t flat;
        int owned = 0;
        int rc = fmm_flatten(p.fmm, p.fmm ? p.levels : 0, &flat, &owned);
        if (rc != FMM_OK) return rc;
        AlgView alg;
        if (host_tables) {
            host_tables->emplace_back();
            rc = fmm_alg_describe(&flat, &host_tables->back(), &alg);
        } else {
            rc = fmm_alg_get(&flat, &alg);
        }
        if (owned) free_fmm(flat);
        if (rc != FMM_OK) return rc;
        if (p.slices == 0) {
            f64_idx.push_back(i);
            f64_alg.push_back(alg);
            continue;
        }
        SplitJob j;
        rc = job_init(j, alg, p.m, p.n, p.k, p.alpha, p.A, p.lda, p.B, p.ldb, p.beta, p.C, p.ldc, p.slices,
                      p.format);
        if (rc != FMM_OK) return rc;
        jobs.push_back(j);
    }
    return FMM_OK;
}

}  // namespace

/* Batch workspace: the FP64 problems' table, then the split problems' region. */
static size_t batch_f64_bytes(size_t nf64) { return nf64 ? fmm_f64_batch_ws_bytes((int)nf64) : 0; }

extern "C" size_t fmm_gpu_batch_workspace_size(int count, const fmm_batch_problem* probs)
{
    std::vector<SplitJob> jobs;
    std::vector<int> fi;
    std::vector<AlgView> fa;
    std::deque<std::vector<int>> tables;
    if (batch_jobs(count, probs, jobs, fi, fa, &tables) != FMM_OK) return 0;
    const size_t split = jobs.empty() ? 0 : fmm_split_batch_ws((int)jobs.size(), jobs.data());
    return std::max<size_t>(256, batch_f64_bytes(fi.size()) + split);
}

extern "C" int fmm_gpu_batch_dgemm(int count, const fmm_batch_problem* probs, void* workspace,
                                   size_t workspace_bytes, void* stream)
{
    std::vector<SplitJob> jobs;
    std::vector<int> fi;
    std::vector<AlgView> fa;
    int rc = batch_jobs(count, probs, jobs, fi, fa);
    if (rc != FMM_OK) return rc;
    if (fmm_device_error_word() == nullptr) return FMM_ERR_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t f64_bytes = batch_f64_bytes(fi.size());
    if (!fi.empty()) {
        /* all FP64 problems in one persistent launch */
        std::vector<F64BatchItem> items(fi.size());
        for (size_t q = 0; q < fi.size(); ++q) {
            const fmm_batch_problem& p = probs[fi[q]];
            items[q] = F64BatchItem{fa[q], p.m, p.n, p.k, p.alpha, p.beta, p.A, p.lda, p.B, p.ldb, p.C, p.ldc};
        }
        rc = fmm_f64_batch_launch((int)items.size(), items.data(), workspace, workspace_bytes, st);
        if (rc != FMM_OK) return rc;
    }
    if (!jobs.empty()) {
        if (workspace_bytes < f64_bytes) return FMM_ERR_WORKSPACE;
        workspace = workspace ? (void*)((uint8_t*)workspace + f64_bytes) : nullptr;
        workspace_bytes -= f64_bytes;
    }
    if (jobs.empty()) return FMM_OK;
    return fmm_split_batch((int)jobs.size(), jobs.data(), workspace, workspace_bytes, st);
}

/* ---------------------------------------------------------------------------
 * Self-test of the failure path every kernel wait relies on: one CTA waits,
 * with the library's bounded mbarrier wait (sm103::mbar_wait, the one the GEMM
 * kernels use), on a barrier that nothing arrives at. After the wait limit it
 * must record `code` in the device error word, raise the CTA's abort flag so
 * the other waiting threads give up too, and return; the kernel then ends
 * normally and the context stays usable.
 * ------------------------------------------------------------------------- */
namespace {
__global__ void __launch_bounds__(64) selftest_wait_kernel(int* err, int code, int* gave_up)
{
    __shared__ uint64_t bar;
    __shared__ volatile int abort_flag;
    if (threadIdx.x == 0) {
        sm103::mbar_init(&bar, 1);     /* one arrival expected; none comes */
        abort_flag = 0;
        sm103::fence_mbar_init();
    }
    __syncthreads();
    const bool ok = sm103::mbar_wait(&bar, 0, &abort_flag, err, code);
    if (!ok) atomicAdd(gave_up, 1);
}
}  // namespace

extern "C" int fmm_gpu_selftest_wait_expiry(int* threads_gave_up)
{
    int* err = fmm_device_error_word();
    if (err == nullptr) return FMM_ERR_CUDA;
    int* d_gave = nullptr;
    if (cudaMalloc(&d_gave, sizeof(int)) != cudaSuccess) return FMM_ERR_ALLOC;
    int rc = FMM_OK;
    if (cudaMemset(d_gave, 0, sizeof(int)) != cudaSuccess) rc = FMM_ERR_CUDA;
    if (rc == FMM_OK) {
        selftest_wait_kernel<<<1, 64>>>(err, 99, d_gave);
        fmm_count_launch(1);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = FMM_ERR_CUDA;
    }
    int gave = 0;
    if (rc == FMM_OK && cudaMemcpy(&gave, d_gave, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) rc = FMM_ERR_CUDA;
    cudaFree(d_gave);
    if (threads_gave_up) *threads_gave_up = gave;
    if (rc != FMM_OK) return rc;
    return fmm_device_error_status();
}

extern "C" void fmm_gpu_set_host_timeline(int enable) { g_timeline.store(enable != 0); }

extern "C" int fmm_gpu_read_host_timeline(double* ms, int count)
{
    if (ms == nullptr || count < 0) return FMM_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_timeline_mu);
    const int c = std::min(count, kTimelinePoints + 1);
    for (int x = 0; x < c; ++x) ms[x] = g_timeline_ms[x];
    return c;
}
