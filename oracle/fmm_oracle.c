/*
 * ORACLE -- test infrastructure only. A CPU restatement of the reference's
 * FMM GEMM path, used by tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline as the checker. Nothing in the shipped library links or calls it.
 *
 * Restates, in plain C with OpenMP:
 *   - the sub-block geometry of frame/base/bli_strassen_ab.c:26-84 (each
 *     product runs at ceil(dim/t) with zero fill) and :86-121 (the first
 *     dim % t blocks have floor+1 elements, the rest floor; offsets are
 *     cumulative);
 *   - the per-product loop of frame/base/bli_strassen_ab.c:248-294, run over
 *     all R products (the reference stops at FMM_BLIS_MULTS = 7, which is only
 *     right for R = 7);
 *   - the fused pack of plugin/ref_kernels/bli_packm_fmm_ref.c:89-147:
 *     S_r = sum_i U[i,r] * A_i in part order, with zero fill past each part;
 *   - the multi-C epilogue of plugin/ref_kernels/bli_gemm_fmm_ref.c:99-120:
 *     C_p += W[p,r] * M_r clipped to part p's size.
 * Scalars: C := beta*C + alpha*A*B with beta applied once and alpha once (the
 * reference applies beta per product and part and alpha twice, so it is only
 * right for alpha = beta = 1, the case every parity test uses).
 * Zero coefficients are skipped (the reference adds 0*x, identical for
 * finite inputs).
 *
 * Also restates the classical triple loop of test/test_strassen_oapi.c:18-42
 * (my_mm, C += A*B) and, for the split-precision form, the exact digit
 * arithmetic the GPU kernels perform (oracle_split_*), so the GPU result can be
 * compared bit for bit.
 *
 * Parity pin: the reference has no golden vectors; its one known-answer test
 * (test/test_strassen_oapi.c:44-242, m=3 n=13 k=7, 222.txt, FMM against the
 * naive loop, Frobenius residual, gate 1e-7) is restated in
 * tests/test_oracle.py together with the Brent equations of every
 * coefficient file.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Sub-block i of a dimension of length d split t ways
 * (frame/base/bli_strassen_ab.c:86-121). */
static void part_geom(int64_t d, int t, int i, int64_t* off, int64_t* len)
{
    int64_t base = d / t, rem = d % t;
    *off = (int64_t)i * base + (i < rem ? i : rem);
    *len = base + (i < rem ? 1 : 0);
}

int oracle_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* C(m x n) += A(m x k) * B(k x n), all column-major, blocked for cache and
 * parallel over column blocks of C. Summation over p runs in increasing p
 * for every element. */
static void gemm_acc(int64_t m, int64_t n, int64_t k,
                     const double* A, int64_t lda, const double* B, int64_t ldb,
                     double* C, int64_t ldc, double alpha)
{
    const int64_t NB = 32, KB = 256, MB = 512;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t j0 = 0; j0 < n; j0 += NB) {
        int64_t j1 = j0 + NB < n ? j0 + NB : n;
        for (int64_t p0 = 0; p0 < k; p0 += KB) {
            int64_t p1 = p0 + KB < k ? p0 + KB : k;
            for (int64_t i0 = 0; i0 < m; i0 += MB) {
                int64_t i1 = i0 + MB < m ? i0 + MB : m;
                for (int64_t j = j0; j < j1; ++j) {
                    double* c = C + j * ldc;
                    for (int64_t p = p0; p < p1; ++p) {
                        double b = alpha * B[p + j * ldb];
                        const double* a = A + p * lda;
                        for (int64_t i = i0; i < i1; ++i) c[i] += a[i] * b;
                    }
                }
            }
        }
    }
}

/* test/test_strassen_oapi.c:18-42: C += A*B, plain triple loop. */
void oracle_naive_dgemm(int64_t m, int64_t n, int64_t k,
                        const double* A, int64_t lda, const double* B, int64_t ldb,
                        double* C, int64_t ldc)
{
    for (int64_t i = 0; i < m; ++i)
        for (int64_t j = 0; j < n; ++j)
            for (int64_t p = 0; p < k; ++p)
                C[i + j * ldc] += A[i + p * lda] * B[p + j * ldb];
}

/* C := beta*C + alpha*A*B, classical, blocked. */
void oracle_dgemm(int64_t m, int64_t n, int64_t k, double alpha,
                  const double* A, int64_t lda, const double* B, int64_t ldb,
                  double beta, double* C, int64_t ldc)
{
    if (beta != 1.0)
        for (int64_t j = 0; j < n; ++j)
            for (int64_t i = 0; i < m; ++i)
                C[i + j * ldc] = beta == 0.0 ? 0.0 : beta * C[i + j * ldc];
    if (m > 0 && n > 0 && k > 0 && alpha != 0.0)
        gemm_acc(m, n, k, A, lda, B, ldb, C, ldc, alpha);
}

/* S(rows x cols, ld = rows) = sum over parts q of coef[q] * part_q, parts of
 * X (an (X_rows x X_cols) matrix split rt x ct) zero filled to rows x cols.
 * Parts are visited in index order, as the packm plugin does. */
static void combine_parts(const double* X, int64_t ldx, int64_t X_rows, int64_t X_cols,
                          int rt, int ct, const int* coef, int coef_stride,
                          double* S, int64_t rows, int64_t cols)
{
    memset(S, 0, sizeof(double) * (size_t)(rows * cols));
    for (int q = 0; q < rt * ct; ++q) {
        int c = coef[(size_t)q * coef_stride];
        if (c == 0) continue;
        int64_t ro, rl, co, cl;
        part_geom(X_rows, rt, q / ct, &ro, &rl);
        part_geom(X_cols, ct, q % ct, &co, &cl);
        const double dc = (double)c;
#pragma omp parallel for schedule(static)
        for (int64_t j = 0; j < cl; ++j) {
            const double* x = X + ro + (co + j) * ldx;
            double* s = S + j * rows;
            for (int64_t i = 0; i < rl; ++i) s[i] += dc * x[i];
        }
    }
}

/* One flat FMM level with products [r_begin, r_end) (all: 0, R).
 * mt, kt, nt, R, U, V, W as in fmm_t (U row q = A block (q/kt, q%kt), ...).
 * beta is applied only when r_begin == 0. Returns 0 or -1 on allocation
 * failure. */
int oracle_fmm_dgemm(int mt, int kt, int nt, int R,
                     const int* U, const int* V, const int* W,
                     int64_t m, int64_t n, int64_t k, double alpha,
                     const double* A, int64_t lda, const double* B, int64_t ldb,
                     double beta, double* C, int64_t ldc,
                     int r_begin, int r_end)
{
    if (r_begin == 0 && beta != 1.0)
        for (int64_t j = 0; j < n; ++j)
            for (int64_t i = 0; i < m; ++i)
                C[i + j * ldc] = beta == 0.0 ? 0.0 : beta * C[i + j * ldc];
    if (m == 0 || n == 0 || k == 0 || alpha == 0.0) return 0;
    const int64_t me = (m + mt - 1) / mt, ke = (k + kt - 1) / kt, ne = (n + nt - 1) / nt;
    double* S = (double*)malloc(sizeof(double) * (size_t)(me * ke));
    double* T = (double*)malloc(sizeof(double) * (size_t)(ke * ne));
    double* M = (double*)malloc(sizeof(double) * (size_t)(me * ne));
    if (!S || !T || !M) { free(S); free(T); free(M); return -1; }
    if (r_end > R) r_end = R;
    for (int r = r_begin; r < r_end; ++r) {
        int any_w = 0;
        for (int p = 0; p < mt * nt; ++p) any_w |= W[(size_t)p * R + r] != 0;
        if (!any_w) continue;
        combine_parts(A, lda, m, k, mt, kt, U + r, R, S, me, ke);
        combine_parts(B, ldb, k, n, kt, nt, V + r, R, T, ke, ne);
        memset(M, 0, sizeof(double) * (size_t)(me * ne));
        gemm_acc(me, ne, ke, S, me, T, ke, M, me, 1.0);
        for (int p = 0; p < mt * nt; ++p) {
            int w = W[(size_t)p * R + r];
            if (w == 0) continue;
            int64_t ro, rl, co, cl;
            part_geom(m, mt, p / nt, &ro, &rl);
            part_geom(n, nt, p % nt, &co, &cl);
            const double lam = alpha * (double)w;
#pragma omp parallel for schedule(static)
            for (int64_t j = 0; j < cl; ++j) {
                double* c = C + ro + (co + j) * ldc;
                const double* mm = M + j * me;
                for (int64_t i = 0; i < rl; ++i) c[i] += lam * mm[i];
            }
        }
    }
    free(S); free(T); free(M);
    return 0;
}

/* ------------------------------------------------------------------------
 * Split-precision form: the exact arithmetic of the GPU kernels restated.
 * Every step is integer arithmetic except the FP64 operand sums (fma in part
 * order), the bounds (fma in the same order), the int64 -> double
 * conversion, the power-of-two scaling and the C update (fma), so the result
 * must match the GPU bit for bit.
 * ---------------------------------------------------------------------- */

static int o_exp_above(double b)
{
    uint64_t bits;
    memcpy(&bits, &b, 8);
    bits &= 0x7fffffffffffffffull;
    if (bits == 0) return 0;
    int bexp = (int)(bits >> 52);
    if (bexp > 0) return bexp - 1022;
    return -1010 - __builtin_clzll(bits);
}

/* Balanced base-2^db digits of x relative to 2^E: X = round(x * 2^(db*s-E-1))
 * (ties away from zero), then digits d[s-1..1] in [-2^(db-1), 2^(db-1)) from
 * the bottom and the rest in d[0]. db = 8: BF16 slices; db = 5: FP8-E4M3. */
static void o_split_digits(double x, int E, int s, int db, int* d)
{
    uint64_t bits;
    memcpy(&bits, &x, 8);
    int neg = (int)(bits >> 63);
    int bexp = (int)((bits >> 52) & 0x7ff);
    uint64_t mant = bits & 0x000fffffffffffffull;
    int ex;
    if (bexp == 0) ex = -1074; else { mant |= 0x0010000000000000ull; ex = bexp - 1075; }
    int sh = ex + db * s - E - 1;
    int64_t X;
    if (mant == 0 || sh < -62) X = 0;
    else if (sh >= 0) X = (int64_t)(mant << sh);
    else X = (int64_t)((mant + (1ull << (-sh - 1))) >> (-sh));
    if (neg) X = -X;
    const int64_t half = (int64_t)1 << (db - 1), mask = ((int64_t)1 << db) - 1;
    for (int t = s - 1; t >= 1; --t) {
        int dd = (int)(((X + half) & mask) - half);
        d[t] = dd;
        X = (X - dd) >> db;
    }
    d[0] = (int)X;
}

static double o_pow2(int e)
{
    uint64_t bits = (uint64_t)(int64_t)(e + 1023) << 52;
    double v;
    memcpy(&v, &bits, 8);
    return v;
}

static double o_scale2(double v, int e)
{
    if (e > 1000) { v *= o_pow2(1000); e -= 1000; }
    else if (e < -1000) { v *= o_pow2(-1000); e += 1000; }
    return v * o_pow2(e);
}

/* C := beta*C + alpha*A*B through the split form with `s` slices: fmt 0 =
 * BF16 digits (base 256, s = 2..8), fmt 1 = FP8-E4M3 digits (base 32,
 * s = 2..12). With a row list, only the listed rows i of the product grid
 * (0 <= i < ceil(m/m~)) are computed: C rows ro_p + i of every C part row p
 * get their final values, the other rows only beta's scaling; the arithmetic
 * of every computed element is the same as without the list (rows do not
 * interact). Returns 0, or -1 on allocation failure / unsupported size. */
static int split_core(int mt, int kt, int nt, int R,
                      const int* U, const int* V, const int* W,
                      int64_t m, int64_t n, int64_t k, double alpha,
                      const double* A, int64_t lda, const double* B, int64_t ldb,
                      double beta, double* C, int64_t ldc, int s, int fmt,
                      const int64_t* rows, int64_t nrows)
{
    if (beta != 1.0)
        for (int64_t j = 0; j < n; ++j)
            for (int64_t i = 0; i < m; ++i)
                C[i + j * ldc] = beta == 0.0 ? 0.0 : beta * C[i + j * ldc];
    if (m == 0 || n == 0 || k == 0 || alpha == 0.0) return 0;
    if (fmt != 0 && fmt != 1) return -1;
    const int db = fmt ? 5 : 8;               /* digit bits */
    if (s < 2 || s > (fmt ? 12 : 8)) return -1;
    const int64_t me_all = (m + mt - 1) / mt, ke = (k + kt - 1) / kt, ne = (n + nt - 1) / nt;
    if (ke > 16384) return -1;
    if (rows)
        for (int64_t x = 0; x < nrows; ++x)
            if (rows[x] < 0 || rows[x] >= me_all) return -1;
    const int64_t me = rows ? nrows : me_all;   /* rows held; row x is grid row ROW(x) */
#define ROW(x) (rows ? rows[(x)] : (x))
    double* amax = (double*)calloc((size_t)(kt * m), sizeof(double));
    double* bmax = (double*)calloc((size_t)(kt * n), sizeof(double));
    int* Er = (int*)malloc(sizeof(int) * (size_t)me);
    int* Fc = (int*)malloc(sizeof(int) * (size_t)ne);
    double* S = (double*)malloc(sizeof(double) * (size_t)(me * ke));
    double* T = (double*)malloc(sizeof(double) * (size_t)(ke * ne));
    int16_t* DA = (int16_t*)malloc(sizeof(int16_t) * (size_t)(s * me * ke)); /* [t][p][i] */
    int16_t* DB = (int16_t*)malloc(sizeof(int16_t) * (size_t)(s * ke * ne)); /* [u][j][p] */
    int64_t* Z = (int64_t*)malloc(sizeof(int64_t) * (size_t)(me * ne));
    /* Z counts in units of level G: BF16 6, or 7 when the padded k is <= 128;
     * FP8 s + 1 up to 10 (exact for s <= 9) */
    const int64_t k_pad = (ke + 63) / 64 * 64;
    const int G = fmt ? (s + 1 < 10 ? s + 1 : 10) : (k_pad <= 128 ? 7 : 6);
    if (!amax || !bmax || !Er || !Fc || !S || !T || !DA || !DB || !Z) {
        free(amax); free(bmax); free(Er); free(Fc); free(S); free(T); free(DA); free(DB); free(Z);
        return -1;
    }
    for (int b = 0; b < kt; ++b) {
        int64_t co, cl;
        part_geom(k, kt, b, &co, &cl);
        for (int64_t i = 0; i < m; ++i) {
            double mx = 0.0;
            for (int64_t c = 0; c < cl; ++c) { double v = fabs(A[i + (co + c) * lda]); if (v > mx) mx = v; }
            amax[b * m + i] = mx;
        }
        for (int64_t j = 0; j < n; ++j) {
            double mx = 0.0;
            for (int64_t p = 0; p < cl; ++p) { double v = fabs(B[co + p + j * ldb]); if (v > mx) mx = v; }
            bmax[b * n + j] = mx;
        }
    }
    for (int r = 0; r < R; ++r) {
        int any_w = 0;
        for (int p = 0; p < mt * nt; ++p) any_w |= W[(size_t)p * R + r] != 0;
        if (!any_w) continue;
        /* exponents from the FP64 bounds, in part order */
        for (int64_t x = 0; x < me; ++x) {
            const int64_t i = ROW(x);
            double bnd = 0.0;
            int first = 1;
            for (int q = 0; q < mt * kt; ++q) {
                int c = U[(size_t)q * R + r];
                if (!c) continue;
                int64_t ro, rl;
                part_geom(m, mt, q / kt, &ro, &rl);
                if (i >= rl) continue;
                double mx = amax[(q % kt) * m + ro + i], ac = fabs((double)c);
                bnd = first ? ac * mx : fma(ac, mx, bnd);
                first = 0;
            }
            Er[x] = o_exp_above(bnd);
        }
        for (int64_t j = 0; j < ne; ++j) {
            double bnd = 0.0;
            int first = 1;
            for (int q = 0; q < kt * nt; ++q) {
                int c = V[(size_t)q * R + r];
                if (!c) continue;
                int64_t co, cl;
                part_geom(n, nt, q % nt, &co, &cl);
                if (j >= cl) continue;
                double mx = bmax[(q / nt) * n + co + j], ac = fabs((double)c);
                bnd = first ? ac * mx : fma(ac, mx, bnd);
                first = 0;
            }
            Fc[j] = o_exp_above(bnd);
        }
        /* operand sums: first nonzero coefficient times its element, then fma */
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < ke; ++p)
            for (int64_t x = 0; x < me; ++x) {
                const int64_t i = ROW(x);
                double sum = 0.0;
                int first = 1;
                for (int q = 0; q < mt * kt; ++q) {
                    int c = U[(size_t)q * R + r];
                    if (!c) continue;
                    int64_t ro, rl, co, cl;
                    part_geom(m, mt, q / kt, &ro, &rl);
                    part_geom(k, kt, q % kt, &co, &cl);
                    double v = (i < rl && p < cl) ? A[ro + i + (co + p) * lda] : 0.0;
                    sum = first ? (double)c * v : fma((double)c, v, sum);
                    first = 0;
                }
                S[x + p * me] = sum;
            }
#pragma omp parallel for schedule(static)
        for (int64_t j = 0; j < ne; ++j)
            for (int64_t p = 0; p < ke; ++p) {
                double sum = 0.0;
                int first = 1;
                for (int q = 0; q < kt * nt; ++q) {
                    int c = V[(size_t)q * R + r];
                    if (!c) continue;
                    int64_t ro, rl, co, cl;
                    part_geom(k, kt, q / nt, &ro, &rl);
                    part_geom(n, nt, q % nt, &co, &cl);
                    double v = (p < rl && j < cl) ? B[ro + p + (co + j) * ldb] : 0.0;
                    sum = first ? (double)c * v : fma((double)c, v, sum);
                    first = 0;
                }
                T[p + j * ke] = sum;
            }
        /* digits */
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < ke; ++p)
            for (int64_t i = 0; i < me; ++i) {
                int d[12];
                o_split_digits(S[i + p * me], Er[i], s, db, d);
                for (int t = 0; t < s; ++t) DA[((size_t)t * ke + p) * me + i] = (int16_t)d[t];
            }
#pragma omp parallel for schedule(static)
        for (int64_t j = 0; j < ne; ++j)
            for (int64_t p = 0; p < ke; ++p) {
                int d[12];
                o_split_digits(T[p + j * ke], Fc[j], s, db, d);
                for (int t = 0; t < s; ++t) DB[((size_t)t * ne + j) * ke + p] = (int16_t)d[t];
            }
        /* level sums folded into Z (units of level G) */
#pragma omp parallel for schedule(static)
        for (int64_t j = 0; j < ne; ++j) {
            int64_t* lv = (int64_t*)malloc(sizeof(int64_t) * (size_t)me);
            for (int64_t i = 0; i < me; ++i) Z[i + j * me] = 0;
            for (int g = 2; g <= s + 1; ++g) {
                for (int64_t i = 0; i < me; ++i) lv[i] = 0;
                for (int t = 1; t <= s; ++t) {
                    int u = g - t;
                    if (u < 1 || u > s) continue;
                    const int16_t* eb = DB + ((size_t)(u - 1) * ne + j) * ke;
                    for (int64_t p = 0; p < ke; ++p) {
                        int64_t e = eb[p];
                        if (!e) continue;
                        const int16_t* da = DA + ((size_t)(t - 1) * ke + p) * me;
                        for (int64_t i = 0; i < me; ++i) lv[i] += (int64_t)da[i] * e;
                    }
                }
                for (int64_t i = 0; i < me; ++i) {
                    if (g <= G) Z[i + j * me] += lv[i] * ((int64_t)1 << (db * (G - g)));
                    else {
                        int sh = db * (g - G);
                        Z[i + j * me] += (lv[i] + ((int64_t)1 << (sh - 1))) >> sh;
                    }
                }
            }
            free(lv);
        }
        /* multi-C epilogue */
        for (int p = 0; p < mt * nt; ++p) {
            int w = W[(size_t)p * R + r];
            if (!w) continue;
            int64_t ro, rl, co, cl;
            part_geom(m, mt, p / nt, &ro, &rl);
            part_geom(n, nt, p % nt, &co, &cl);
            double lam = alpha * (double)w;
            for (int64_t j = 0; j < cl; ++j)
                for (int64_t x = 0; x < me; ++x) {
                    const int64_t i = ROW(x);
                    if (i >= rl) continue;
                    double v = o_scale2((double)Z[x + j * me], Er[x] + Fc[j] + 2 - db * G);
                    double* c = C + ro + i + (co + j) * ldc;
                    *c = fma(lam, v, *c);
                }
        }
    }
#undef ROW
    free(amax); free(bmax); free(Er); free(Fc); free(S); free(T); free(DA); free(DB); free(Z);
    return 0;
}

int oracle_split_fmm_dgemm_fmt(int mt, int kt, int nt, int R,
                               const int* U, const int* V, const int* W,
                               int64_t m, int64_t n, int64_t k, double alpha,
                               const double* A, int64_t lda, const double* B, int64_t ldb,
                               double beta, double* C, int64_t ldc, int s, int fmt)
{
    return split_core(mt, kt, nt, R, U, V, W, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, s, fmt, NULL, 0);
}

/* The split form on the listed rows of the product grid only (see split_core). */
int oracle_split_fmm_dgemm_rows(int mt, int kt, int nt, int R,
                                const int* U, const int* V, const int* W,
                                int64_t m, int64_t n, int64_t k, double alpha,
                                const double* A, int64_t lda, const double* B, int64_t ldb,
                                double beta, double* C, int64_t ldc, int s, int fmt,
                                const int64_t* rows, int64_t nrows)
{
    if (rows == NULL || nrows <= 0) return -1;
    return split_core(mt, kt, nt, R, U, V, W, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, s, fmt, rows, nrows);
}

/* BF16 split form (fmt 0) */
int oracle_split_fmm_dgemm(int mt, int kt, int nt, int R,
                           const int* U, const int* V, const int* W,
                           int64_t m, int64_t n, int64_t k, double alpha,
                           const double* A, int64_t lda, const double* B, int64_t ldb,
                           double beta, double* C, int64_t ldc, int s)
{
    return oracle_split_fmm_dgemm_fmt(mt, kt, nt, R, U, V, W, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, s, 0);
}
