/*
 * Plain FP64 form of the FMM GEMM (and, with the trivial algorithm, the
 * classical FP64 GEMM it is compared against).
 *
 * On GB300 the FP64 pipe delivers about 2 FMA/clock/SM (1.2 TFLOP/s on the
 * GPU; the FP64 mma.sync path measures slightly slower), so this form is
 * bound by FP64 FMAs and everything else is arranged to cost few of them:
 *
 *  - one CTA owns an output tile position (ti, tj) of the ceil(m/m~) x
 *    ceil(n/n~) product grid and runs every product r over it, so a C
 *    sub-block tile is only ever updated by its owning CTA: no atomics, a
 *    fixed summation order, one launch for the whole algorithm;
 *  - per k step it loads the nnz(U[:,r]) A sub-block tiles and nnz(V[:,r]) B
 *    sub-block tiles straight from the caller's column-major matrices with
 *    coalesced loads, forms the weighted sums in FP64 in registers (the fused
 *    multi-operand pack, plugin/ref_kernels/bli_packm_fmm_ref.c:89-147, with
 *    zero fill past a smaller sub-block as in :133-134) and stores the
 *    combined operand tiles to shared memory;
 *  - a register-blocked DFMA micro-kernel multiplies the tiles (in place of
 *    bli_dgemm_haswell_asm_6x8 called at plugin/ref_kernels/bli_gemm_fmm_ref.c:85-97);
 *  - the k loop stays in registers, and the epilogue adds alpha*W[p,r]*tile
 *    into every C sub-block p with W[p,r] != 0, clipped to its size
 *    (bli_gemm_fmm_ref.c:99-120), with one coalesced read-modify-write per
 *    (product, sub-block) instead of one per KC block.
 */
#include "fmm_internal.h"

#include <cooperative_groups.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <vector>

namespace cg = cooperative_groups;

/* k chunks of the small/skinny classical path for an m x n x k FP64
 * problem, 0 when the regular kernel runs it: at most 128 output tiles of
 * 32 x 32, chunks of at least 256 k, at most 8 chunks (a portable cluster)
 * and at most 256 CTAs. A function of the shape only, so single and batched
 * calls take the same path. */
extern "C" int fmm_gpu_f64_sup_splits(int64_t m, int64_t n, int64_t k)
{
    if (m <= 0 || n <= 0 || k <= 0) return 0;
    const int64_t tiles = ((m + 31) / 32) * ((n + 31) / 32);
    if (tiles > 128) return 0;
    const int64_t ks = std::min<int64_t>({8, 256 / tiles, k / 256});
    return ks >= 2 ? (int)ks : 0;
}

/* chunk length: k / ks rounded up to whole 32-k steps; every chunk is
 * non-empty because each holds at least 256 k */
int64_t fmm_f64_sup_chunk(int64_t k, int ks)
{
    return ((k + ks - 1) / ks + 31) / 32 * 32;
}

namespace {

constexpr int kMaxEntries = 256;  /* nonzero coefficients per product column */

/* micro-kernel of the plain form (fmm_gpu_set_f64_engine): FMM_F64_DFMA or FMM_F64_MMA */
std::atomic<int> g_f64_engine{FMM_F64_DFMA};

struct Entry {
    const double* base;  /* sub-block origin in the source matrix */
    double coef;         /* small integer coefficient, already a double */
    int rows, cols;      /* sub-block extent */
    int kind;            /* 0: +1, 1: -1, 2: other (no FP64 compare per element) */
    int pad;
};

/* first term of a combination: s[t] = c * v[t], exact like the FP64
 * product; sign flips for c = +-1 keep it off the FP64 pipe that the
 * micro-kernel is bound by. One uniform branch for all of a thread's values. */
template <int N>
__device__ __forceinline__ void scale_first(const Entry& x, double (&s)[N])
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

/* Geometry of the nonzero entries [beg, end) of one product column of U
 * (or V), for a source split rt x ct, into shared memory. */
__device__ void stage_entries(const int* __restrict__ ent, int beg, int end, int ct,
                              int rt, const double* src, int64_t ld, int64_t rows_total,
                              int64_t cols_total, Entry* out)
{
    for (int e = beg + (int)threadIdx.x; e < end; e += blockDim.x) {
        int part = ent[2 * e], coef = ent[2 * e + 1];
        int64_t ro, rl, co, cl;
        fmm_part_geom(rows_total, rt, part / ct, &ro, &rl);
        fmm_part_geom(cols_total, ct, part % ct, &co, &cl);
        Entry x;
        x.base = src + ro + co * ld;
        x.rows = (int)rl;
        x.cols = (int)cl;
        x.coef = (double)coef;
        x.kind = coef == 1 ? 0 : (coef == -1 ? 1 : 2);
        x.pad = 0;
        out[e - beg] = x;
    }
}

/* One output tile position (ti, tj) of the ceil(m/m~) x ceil(n/n~) product
 * grid: every product r of the algorithm over it, with the fused packs, the
 * DFMA micro-kernel and the multi-C epilogue. Shared by the single-problem
 * kernel (one CTA per tile position) and the batched one (a work queue of
 * (problem, tile position) items). */
/* Shared-memory layout of the combined operand tiles. DFMA engine: A as
 * [k][m] and B as [k][n], pitch +1 (the micro-kernel reads a row of each).
 * FP64 MMA engine: A as [k][m] with pitch BM + 8 and B transposed to [n][k]
 * with pitch BK + 4, so both the fused packs' stores (consecutive m, or
 * consecutive k) and the m8n8k4 fragment loads (A[gid][tig], B[tig][gid])
 * hit distinct banks. */
template <int BM, int BN, int BK, bool MMA>
struct F64Smem {
    static constexpr int PA = MMA ? BM + 8 : BM + 1;
    static constexpr int PB = MMA ? BK + 4 : BN + 1;
    static constexpr int A_ELEMS = BK * PA;
    static constexpr int B_ELEMS = MMA ? BN * PB : BK * PB;
    __device__ static __forceinline__ int a(int kk, int mm) { return kk * PA + mm; }
    __device__ static __forceinline__ int b(int kk, int nn) { return MMA ? nn * PB + kk : kk * PB + nn; }
};

/* D += A * B on an 8 x 8 x 4 FP64 tile, one warp (mma.sync.m8n8k4.f64):
 * a = A[gid][tig], b = B[tig][gid], d = D[gid][2 tig .. 2 tig + 1] with
 * gid = lane / 4, tig = lane % 4. */
__device__ __forceinline__ void mma_f64_8x8x4(double (&d)[2], double a, double b)
{
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                 : "+d"(d[0]), "+d"(d[1])
                 : "d"(a), "d"(b));
}

template <int BM, int BN, int BK, int TM, int TN, bool MMA>
__device__ __forceinline__ void f64_tile(const int* __restrict__ tab, int64_t m, int64_t n, int64_t k,
                                         double alpha, const double* __restrict__ A, int64_t lda,
                                         const double* __restrict__ B, int64_t ldb,
                                         double* __restrict__ C, int64_t ldc, int ti, int tj,
                                         double* As, double* Bs,
                                         Entry* ue, Entry* ve, int r_begin, int r_end,
                                         const double* __restrict__ Sp, const double* __restrict__ Tp)
{
    using SM = F64Smem<BM, BN, BK, MMA>;
    constexpr int NT = (BM / TM) * (BN / TN);
    constexpr int RT = BM / TM;  /* thread rows */
    constexpr int CT = BN / TN;  /* thread cols */
    static_assert(NT % BM == 0 && NT % BK == 0, "tile/thread mapping");

    const int mt = tab[0], kt = tab[1], nt = tab[2], R = tab[3];
    const int* u_off = tab + FMM_ALG_HDR;
    const int* v_off = u_off + (R + 1);
    const int* w_off = v_off + (R + 1);
    const int* ents = w_off + (R + 1);          /* (part, coef) pairs */
    const int* u_ent = ents;
    const int* v_ent = ents + 2 * u_off[R];
    const int* w_ent = v_ent + 2 * v_off[R];

    const int64_t me = (m + mt - 1) / mt, ne = (n + nt - 1) / nt, ke = (k + kt - 1) / kt;
    const int64_t i0 = (int64_t)ti * BM, j0 = (int64_t)tj * BN;
    const int tid = threadIdx.x;
    const int tr = tid % RT, tc = tid / RT;
    /* With pre-formed operands (Sp/Tp: S_r, T_r of the products r_begin..,
     * me x ke and ke x ne column-major) every product has one term of
     * coefficient 1, read with those strides; its values are exactly what the
     * fused pack forms. */
    if (Sp) { lda = me; ldb = ke; }
    (void)R;

    for (int r = r_begin; r < r_end; ++r) {
        const int wb = w_off[r], we = w_off[r + 1];
        if (wb == we) continue;
        int ue_n, ve_n;
        __syncthreads();  /* previous product finished with ue/ve */
        if (Sp) {
            ue_n = ve_n = 1;
            if (tid == 0) {
                ue[0] = Entry{Sp + (int64_t)(r - r_begin) * me * ke, 1.0, (int)me, (int)ke, 0, 0};
                ve[0] = Entry{Tp + (int64_t)(r - r_begin) * ke * ne, 1.0, (int)ke, (int)ne, 0, 0};
            }
        } else {
            const int ub = u_off[r], vb = v_off[r];
            ue_n = u_off[r + 1] - ub;
            ve_n = v_off[r + 1] - vb;
            stage_entries(u_ent, ub, ub + ue_n, kt, mt, A, lda, m, k, ue);
            stage_entries(v_ent, vb, vb + ve_n, nt, kt, B, ldb, k, n, ve);
        }
        __syncthreads();

        /* MMA engine: 8 warps in a WGM x (8 / WGM) grid, each an (MB*8) x (NB*8) block of fragments */
        constexpr int WGM = BM >= 64 ? BM / 32 : 4;
        constexpr int WM = BM / WGM, WN = BN / (8 / WGM);
        constexpr int MB = MMA ? WM / 8 : 1, NB = MMA ? WN / 8 : 1;
        static_assert(!MMA || (NT == 256 && WM % 8 == 0 && WN % 8 == 0 && BK % 4 == 0), "MMA warp tiling");
        const int lane = tid % 32, wid = tid / 32, gid = lane / 4, tig = lane % 4;
        const int wm = wid % WGM, wn = wid / WGM;
        double acc[MMA ? 1 : TM][MMA ? 1 : TN];
        double facc[MB][NB][2];
        if (MMA) {
#pragma unroll
            for (int a = 0; a < MB; ++a)
#pragma unroll
                for (int b = 0; b < NB; ++b) facc[a][b][0] = facc[a][b][1] = 0.0;
        } else {
#pragma unroll
            for (int a = 0; a < (MMA ? 1 : TM); ++a)
#pragma unroll
                for (int b = 0; b < (MMA ? 1 : TN); ++b) acc[a][b] = 0.0;
        }

        for (int64_t k0 = 0; k0 < ke; k0 += BK) {
            /* fused pack of the A-side combination: BM x BK. Each term's
             * loads for all of this thread's elements go out together; the
             * first term's coefficient (uniform over the CTA) is applied once
             * after them. */
            {
                constexpr int NA = BM * BK / NT;
                const int li = tid % BM;
                const int64_t gi = i0 + li;
                double s[NA];
#pragma unroll
                for (int t = 0; t < NA; ++t) s[t] = 0.0;
                if (ue_n > 0) {
                    const Entry& x0 = ue[0];
#pragma unroll
                    for (int t = 0; t < NA; ++t) {
                        const int64_t gp = k0 + tid / BM + t * (NT / BM);
                        s[t] = (gi < x0.rows && gp < x0.cols) ? x0.base[gi + gp * lda] : 0.0;
                    }
                    scale_first(x0, s);
                }
                for (int e = 1; e < ue_n; ++e) {
                    const Entry& x = ue[e];
#pragma unroll
                    for (int t = 0; t < NA; ++t) {
                        const int64_t gp = k0 + tid / BM + t * (NT / BM);
                        const double v = (gi < x.rows && gp < x.cols) ? x.base[gi + gp * lda] : 0.0;
                        s[t] = fma(x.coef, v, s[t]);
                    }
                }
#pragma unroll
                for (int t = 0; t < NA; ++t) As[SM::a(tid / BM + t * (NT / BM), li)] = s[t];
            }
            /* fused pack of the B-side combination: BK x BN */
            {
                constexpr int NB = BK * BN / NT;
                const int lp = tid % BK;
                const int64_t gp = k0 + lp;
                double s[NB];
#pragma unroll
                for (int t = 0; t < NB; ++t) s[t] = 0.0;
                if (ve_n > 0) {
                    const Entry& x0 = ve[0];
#pragma unroll
                    for (int t = 0; t < NB; ++t) {
                        const int64_t gj = j0 + tid / BK + t * (NT / BK);
                        s[t] = (gp < x0.rows && gj < x0.cols) ? x0.base[gp + gj * ldb] : 0.0;
                    }
                    scale_first(x0, s);
                }
                for (int e = 1; e < ve_n; ++e) {
                    const Entry& x = ve[e];
#pragma unroll
                    for (int t = 0; t < NB; ++t) {
                        const int64_t gj = j0 + tid / BK + t * (NT / BK);
                        const double v = (gp < x.rows && gj < x.cols) ? x.base[gp + gj * ldb] : 0.0;
                        s[t] = fma(x.coef, v, s[t]);
                    }
                }
#pragma unroll
                for (int t = 0; t < NB; ++t) Bs[SM::b(lp, tid / BK + t * (NT / BK))] = s[t];
            }
            __syncthreads();
            if (MMA) {
#pragma unroll 2
                for (int kk = 0; kk < BK; kk += 4) {
                    double a[MB], b[NB];
#pragma unroll
                    for (int x = 0; x < MB; ++x) a[x] = As[SM::a(kk + tig, wm * WM + x * 8 + gid)];
#pragma unroll
                    for (int y = 0; y < NB; ++y) b[y] = Bs[SM::b(kk + tig, wn * WN + y * 8 + gid)];
#pragma unroll
                    for (int x = 0; x < MB; ++x)
#pragma unroll
                        for (int y = 0; y < NB; ++y) mma_f64_8x8x4(facc[x][y], a[x], b[y]);
                }
            } else {
#pragma unroll 4
                for (int kk = 0; kk < BK; ++kk) {
                    double a[MMA ? 1 : TM], b[MMA ? 1 : TN];
#pragma unroll
                    for (int x = 0; x < (MMA ? 1 : TM); ++x) a[x] = As[SM::a(kk, tr + x * RT)];
#pragma unroll
                    for (int y = 0; y < (MMA ? 1 : TN); ++y) b[y] = Bs[SM::b(kk, tc + y * CT)];
#pragma unroll
                    for (int x = 0; x < (MMA ? 1 : TM); ++x)
#pragma unroll
                        for (int y = 0; y < (MMA ? 1 : TN); ++y) acc[x][y] = fma(a[x], b[y], acc[x][y]);
                }
            }
            __syncthreads();
        }

        /* multi-C epilogue */
        for (int e = wb; e < we; ++e) {
            const int part = w_ent[2 * e];
            const double lam = alpha * (double)w_ent[2 * e + 1];
            int64_t ro, rl, co, cl;
            fmm_part_geom(m, mt, part / nt, &ro, &rl);
            fmm_part_geom(n, nt, part % nt, &co, &cl);
            double* cb = C + ro + co * ldc;
            if (MMA) {
#pragma unroll
                for (int y = 0; y < NB; ++y)
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int64_t gj = j0 + wn * WN + y * 8 + 2 * tig + h;
                        if (gj >= cl) continue;
#pragma unroll
                        for (int x = 0; x < MB; ++x) {
                            const int64_t gi = i0 + wm * WM + x * 8 + gid;
                            if (gi < rl) {
                                double* p = cb + gi + gj * ldc;
                                *p = fma(lam, facc[x][y][h], *p);
                            }
                        }
                    }
            } else {
#pragma unroll
                for (int y = 0; y < (MMA ? 1 : TN); ++y) {
                    const int64_t gj = j0 + tc + y * CT;
                    if (gj >= cl) continue;
#pragma unroll
                    for (int x = 0; x < (MMA ? 1 : TM); ++x) {
                        const int64_t gi = i0 + tr + x * RT;
                        if (gi < rl) {
                            double* p = cb + gi + gj * ldc;
                            *p = fma(lam, acc[x][y], *p);
                        }
                    }
                }
            }
        }
    }
    (void)me; (void)ne;
}

template <int BM, int BN, int BK, int TM, int TN, bool MMA>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
fmm_f64_kernel(const int* __restrict__ tab, int64_t m, int64_t n, int64_t k,
               double alpha, const double* __restrict__ A, int64_t lda,
               const double* __restrict__ B, int64_t ldb,
               double* __restrict__ C, int64_t ldc, int tiles_m, int r_begin, int r_end,
               const double* __restrict__ Sp, const double* __restrict__ Tp)
{
    using SM = F64Smem<BM, BN, BK, MMA>;
    __shared__ double As[SM::A_ELEMS];
    __shared__ double Bs[SM::B_ELEMS];
    __shared__ Entry ue[kMaxEntries];
    __shared__ Entry ve[kMaxEntries];
    f64_tile<BM, BN, BK, TM, TN, MMA>(tab, m, n, k, alpha, A, lda, B, ldb, C, ldc, (int)(blockIdx.x % tiles_m),
                                      (int)(blockIdx.x / tiles_m), As, Bs, ue, ve, r_begin, r_end, Sp, Tp);
}

/* ------------------------------------------------------------ batched -- */

/* One problem of a batched FP64 launch; problems are laid out in the order
 * their work items are handed out (item_begin increasing). */
struct F64Prob {
    const int* tab;
    int64_t m, n, k;
    double alpha, beta;
    const double* A;
    int64_t lda;
    const double* B;
    int64_t ldb;
    double* C;
    int64_t ldc;
    int64_t item_begin;   /* first (tile position) item of this problem */
    int tiles_m, tiles_n;
};

constexpr int kF64Bm = 64, kF64Bn = 64, kF64Bk = 32, kF64Tm = 4, kF64Tn = 4;
constexpr int kF64TableChunk = 256;   /* problems per table-writer launch (parameter space) */

struct F64TableChunk {
    F64Prob* dst;
    int count;
    F64Prob p[kF64TableChunk];
};

/* copies a chunk of the problem table (passed by value, so a captured graph
 * holds it) into device memory */
__global__ void f64_table_write(const __grid_constant__ F64TableChunk c)
{
    for (int i = threadIdx.x; i < c.count; i += blockDim.x) c.dst[i] = c.p[i];
}

/* Batched FP64 FMM GEMM: one persistent launch over all (problem, tile
 * position) items of a batch. A CTA takes the next item from an atomic
 * counter (problems sorted by per-item work, largest first, so the long
 * items go out first), applies beta to the C elements its threads own in
 * every sub-block of that tile position, then runs the tile exactly as the
 * single-problem kernel does, so each result is identical to the problem
 * issued alone. */
template <bool MMA>
__global__ void __launch_bounds__((kF64Bm / kF64Tm) * (kF64Bn / kF64Tn))
fmm_f64_batch_kernel(const F64Prob* __restrict__ probs, int nprob, int64_t nitems,
                     unsigned long long* __restrict__ counter)
{
    constexpr int RT = kF64Bm / kF64Tm, CT = kF64Bn / kF64Tn;
    using SM = F64Smem<kF64Bm, kF64Bn, kF64Bk, MMA>;
    __shared__ double As[SM::A_ELEMS];
    __shared__ double Bs[SM::B_ELEMS];
    __shared__ Entry ue[kMaxEntries];
    __shared__ Entry ve[kMaxEntries];
    __shared__ long long next;
    const int tid = threadIdx.x, tr = tid % RT, tc = tid / RT;
    for (;;) {
        __syncthreads();   /* the previous item is done with next, ue and ve */
        if (tid == 0) next = (long long)atomicAdd(counter, 1ull);
        __syncthreads();
        const int64_t b = next;
        if (b >= nitems) break;
        int lo = 0, hi = nprob - 1;        /* last problem with item_begin <= b */
        while (lo < hi) {
            const int mid = (lo + hi + 1) / 2;
            if (probs[mid].item_begin <= b) lo = mid; else hi = mid - 1;
        }
        const F64Prob P = probs[lo];
        const int64_t local = b - P.item_begin;
        const int ti = (int)(local % P.tiles_m), tj = (int)(local / P.tiles_m);
        const int mt = P.tab[0], nt = P.tab[2];
        if (P.beta != 1.0) {
            for (int part = 0; part < mt * nt; ++part) {
                int64_t ro, rl, co, cl;
                fmm_part_geom(P.m, mt, part / nt, &ro, &rl);
                fmm_part_geom(P.n, nt, part % nt, &co, &cl);
                for (int y = 0; y < kF64Tn; ++y) {
                    const int64_t gj = (int64_t)tj * kF64Bn + tc + y * CT;
                    if (gj >= cl) continue;
                    for (int x = 0; x < kF64Tm; ++x) {
                        const int64_t gi = (int64_t)ti * kF64Bm + tr + x * RT;
                        if (gi < rl) {
                            double* q = P.C + ro + gi + (co + gj) * P.ldc;
                            *q = P.beta == 0.0 ? 0.0 : P.beta * *q;
                        }
                    }
                }
            }
        }
        if (P.k == 0 || P.alpha == 0.0) continue;
        f64_tile<kF64Bm, kF64Bn, kF64Bk, kF64Tm, kF64Tn, MMA>(P.tab, P.m, P.n, P.k, P.alpha, P.A, P.lda, P.B, P.ldb,
                                                        P.C, P.ldc, ti, tj, As, Bs, ue, ve, 0, P.tab[3],
                                                        nullptr, nullptr);
    }
}

/* Pre-formed operand combinations for the products r0 .. r0+np-1:
 * S[q][i + p*me] = sum_e U[e,r] A_e[i,p] (A side) or T[q][p + j*ke] =
 * sum_e V[e,r] B_e[p,j] (B side), zero past a smaller sub-block, summed
 * exactly as the fused pack does (the first term's coefficient, then FMAs in
 * entry order), so the GEMM over them gives the fused kernel's bits. One
 * thread per element down a column (coalesced loads and stores); the product
 * index runs fastest in the block order so the products at one position read
 * their shared sub-blocks through L2 once. */
template <bool A_SIDE>
__global__ void __launch_bounds__(256)
f64_combine_kernel(const int* __restrict__ tab, int r0, int np, const double* __restrict__ X, int64_t ldx,
                   int64_t m, int64_t n, int64_t k, double* __restrict__ out)
{
    __shared__ Entry ent[kMaxEntries];
    const int mt = tab[0], kt = tab[1], nt = tab[2], R = tab[3];
    const int* u_off = tab + FMM_ALG_HDR;
    const int* v_off = u_off + (R + 1);
    const int* w_off = v_off + (R + 1);
    const int* u_ent = w_off + (R + 1);
    const int* v_ent = u_ent + 2 * u_off[R];
    const int64_t me = (m + mt - 1) / mt, ne = (n + nt - 1) / nt, ke = (k + kt - 1) / kt;
    const int64_t rows = A_SIDE ? me : ke, cols = A_SIDE ? ke : ne;
    const int q = (int)(blockIdx.x % (unsigned)np), r = r0 + q;
    const int64_t i = (int64_t)(blockIdx.x / (unsigned)np) * blockDim.x + threadIdx.x;
    int ne_;
    if (A_SIDE) {
        ne_ = u_off[r + 1] - u_off[r];
        stage_entries(u_ent, u_off[r], u_off[r + 1], kt, mt, X, ldx, m, k, ent);
    } else {
        ne_ = v_off[r + 1] - v_off[r];
        stage_entries(v_ent, v_off[r], v_off[r + 1], nt, kt, X, ldx, k, n, ent);
    }
    __syncthreads();
    if (i >= rows) return;
    double* o = out + (int64_t)q * rows * cols;
    for (int64_t c = blockIdx.y; c < cols; c += gridDim.y) {
        double sv[1] = {0.0};
        if (ne_ > 0) {
            const Entry& x0 = ent[0];
            sv[0] = (i < x0.rows && c < x0.cols) ? x0.base[i + c * ldx] : 0.0;
            scale_first(x0, sv);
        }
        for (int e = 1; e < ne_; ++e) {
            const Entry& x = ent[e];
            const double v = (i < x.rows && c < x.cols) ? x.base[i + c * ldx] : 0.0;
            sv[0] = fma(x.coef, v, sv[0]);
        }
        o[i + c * rows] = sv[0];
    }
}

__global__ void scale_c_kernel(int64_t m, int64_t n, double beta, double* C, int64_t ldc)
{
    const int64_t total = m * n;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx % m, j = idx / m;
        double* p = C + i + j * ldc;
        *p = beta == 0.0 ? 0.0 : beta * *p;
    }
}

/* ------------------------------------------- small/skinny classical ---- */

/* The classical FP64 GEMM of a small output (at most 128 tiles of 32 x 32)
 * with a long k (the BLIS "sup" shapes, blis/kernels/haswell/3/sup): the
 * regular kernel would run one CTA per tile down the whole of k on a few
 * SMs. Here a cluster of ks CTAs (one per k chunk of kc elements) computes
 * each tile: every CTA accumulates its chunk in k order with the DFMA
 * micro-kernel, leaves its partial tile in shared memory, and after a cluster
 * barrier each CTA sums a share of the tile's elements over the ks partials
 * through distributed shared memory, always in chunk order
 * (((p_0 + p_1) + p_2) + ...), and applies C := fma(alpha, sum, C). The
 * result depends only on (m, n, k): the batched call runs these problems
 * through the same kernel. */
constexpr int kSupB = 32, kSupBk = 32, kSupT = 2, kSupThreads = (kSupB / kSupT) * (kSupB / kSupT);
constexpr int kSupMaxTiles = 128, kSupMaxSplits = 8, kSupMinChunk = 256;

__global__ void __launch_bounds__(kSupThreads)
fmm_f64_sup_kernel(int64_t m, int64_t n, int64_t k, double alpha, const double* __restrict__ A, int64_t lda,
                   const double* __restrict__ B, int64_t ldb, double* __restrict__ C, int64_t ldc, int tiles_m,
                   int ks, int64_t kc)
{
    constexpr int RT = kSupB / kSupT;   /* thread rows (and columns) */
    __shared__ double As[kSupBk][kSupB + 1];
    __shared__ double Bs[kSupBk][kSupB + 1];
    __shared__ double Ps[kSupB * kSupB];          /* this CTA's partial tile, element i + 32 j */
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();        /* the k chunk */
    const int tile = (int)(blockIdx.x / (unsigned)ks);
    const int64_t i0 = (int64_t)(tile % tiles_m) * kSupB, j0 = (int64_t)(tile / tiles_m) * kSupB;
    const int64_t kb = (int64_t)rank * kc, kend = kb + kc < k ? kb + kc : k;
    const int tid = threadIdx.x, tr = tid % RT, tc = tid / RT;
    double acc[kSupT][kSupT];
#pragma unroll
    for (int x = 0; x < kSupT; ++x)
#pragma unroll
        for (int y = 0; y < kSupT; ++y) acc[x][y] = 0.0;
    for (int64_t k0 = kb; k0 < kend; k0 += kSupBk) {
        /* A: 32 rows x 32 k, B: 32 k x 32 columns, zero past the edges */
#pragma unroll
        for (int t = 0; t < kSupB * kSupBk / kSupThreads; ++t) {
            const int e = tid + t * kSupThreads;
            const int li = e % kSupB, lk = e / kSupB;
            const int64_t gi = i0 + li, gk = k0 + lk;
            As[lk][li] = (gi < m && gk < kend) ? __ldg(A + gi + gk * lda) : 0.0;
            const int lk2 = e % kSupBk, lj = e / kSupBk;
            const int64_t gk2 = k0 + lk2, gj = j0 + lj;
            Bs[lk2][lj] = (gk2 < kend && gj < n) ? __ldg(B + gk2 + gj * ldb) : 0.0;
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < kSupBk; ++kk) {
            double a[kSupT], b[kSupT];
#pragma unroll
            for (int x = 0; x < kSupT; ++x) a[x] = As[kk][tr + x * RT];
#pragma unroll
            for (int y = 0; y < kSupT; ++y) b[y] = Bs[kk][tc + y * RT];
#pragma unroll
            for (int x = 0; x < kSupT; ++x)
#pragma unroll
                for (int y = 0; y < kSupT; ++y) acc[x][y] = fma(a[x], b[y], acc[x][y]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int x = 0; x < kSupT; ++x)
#pragma unroll
        for (int y = 0; y < kSupT; ++y) Ps[(tr + x * RT) + kSupB * (tc + y * RT)] = acc[x][y];
    cl.sync();   /* every partial tile of the cluster is in place */
    /* the tile's 1024 elements in groups of 256, group g summed by CTA g % ks */
    for (int g = rank; g < kSupB * kSupB / kSupThreads; g += ks) {
        const int e = g * kSupThreads + tid;
        double s = *cl.map_shared_rank(Ps + e, 0);
        for (int q = 1; q < ks; ++q) s = s + *cl.map_shared_rank(Ps + e, q);
        const int64_t gi = i0 + e % kSupB, gj = j0 + e / kSupB;
        if (gi < m && gj < n) {
            double* p = C + gi + gj * ldc;
            *p = fma(alpha, s, *p);
        }
    }
    cl.sync();   /* no CTA leaves while another still reads its partial */
}

/* the trivial 1 x 1 x 1 algorithm with all three coefficients +1: the
 * classical GEMM C += alpha * A * B */
bool plain_classical(const AlgView& alg)
{
    if (alg.R != 1 || alg.mt != 1 || alg.kt != 1 || alg.nt != 1 || alg.htab == nullptr) return false;
    const int* t = alg.htab;
    const int* u_off = t + FMM_ALG_HDR;
    const int* v_off = u_off + 2;
    const int* w_off = v_off + 2;
    const int* u_ent = w_off + 2;
    const int* v_ent = u_ent + 2 * u_off[1];
    const int* w_ent = v_ent + 2 * v_off[1];
    return u_off[1] == 1 && v_off[1] == 1 && w_off[1] == 1 && u_ent[1] == 1 && v_ent[1] == 1 && w_ent[1] == 1;
}

int sup_launch(int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda, const double* B,
               int64_t ldb, double* C, int64_t ldc, int ks, cudaStream_t st)
{
    const int64_t tm = (m + kSupB - 1) / kSupB, tn = (n + kSupB - 1) / kSupB;
    const int64_t kc = fmm_f64_sup_chunk(k, ks);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(tm * tn * ks));
    cfg.blockDim = dim3(kSupThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)ks;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, fmm_f64_sup_kernel, m, n, k, alpha, A, lda, B, ldb, C, ldc,
                                             (int)tm, ks, kc);
    fmm_count_launch(1);
    return e == cudaSuccess && cudaGetLastError() == cudaSuccess ? FMM_OK : FMM_ERR_CUDA;
}

template <int BM, int BN, int BK, int TM, int TN>
int launch_cfg(const AlgView& alg, int64_t m, int64_t n, int64_t k, double alpha,
               const double* A, int64_t lda, const double* B, int64_t ldb, double* C,
               int64_t ldc, int r_begin, int r_end, const double* Sp, const double* Tp, cudaStream_t st)
{
    const int64_t me = (m + alg.mt - 1) / alg.mt, ne = (n + alg.nt - 1) / alg.nt;
    const int64_t tm = (me + BM - 1) / BM, tn = (ne + BN - 1) / BN;
    if (tm * tn > 0x7fffffffLL) return FMM_ERR_UNSUPPORTED;
    if (g_f64_engine.load(std::memory_order_relaxed) == FMM_F64_MMA)
        fmm_f64_kernel<BM, BN, BK, TM, TN, true><<<(unsigned)(tm * tn), (BM / TM) * (BN / TN), 0, st>>>(
            alg.tab, m, n, k, alpha, A, lda, B, ldb, C, ldc, (int)tm, r_begin, r_end, Sp, Tp);
    else
        fmm_f64_kernel<BM, BN, BK, TM, TN, false><<<(unsigned)(tm * tn), (BM / TM) * (BN / TN), 0, st>>>(
            alg.tab, m, n, k, alpha, A, lda, B, ldb, C, ldc, (int)tm, r_begin, r_end, Sp, Tp);
    fmm_count_launch(1);
    return cudaGetLastError() == cudaSuccess ? FMM_OK : FMM_ERR_CUDA;
}

int launch_pick(int pick, const AlgView& alg, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
                int64_t lda, const double* B, int64_t ldb, double* C, int64_t ldc, int r_begin, int r_end,
                const double* Sp, const double* Tp, cudaStream_t st)
{
    switch (pick) {
    case 3: return launch_cfg<64, 64, 32, 4, 4>(alg, m, n, k, alpha, A, lda, B, ldb, C, ldc, r_begin, r_end, Sp, Tp, st);
    case 4: return launch_cfg<128, 64, 16, 8, 4>(alg, m, n, k, alpha, A, lda, B, ldb, C, ldc, r_begin, r_end, Sp, Tp, st);
    case 5: return launch_cfg<64, 128, 16, 4, 8>(alg, m, n, k, alpha, A, lda, B, ldb, C, ldc, r_begin, r_end, Sp, Tp, st);
    default: return launch_cfg<32, 32, 32, 2, 2>(alg, m, n, k, alpha, A, lda, B, ldb, C, ldc, r_begin, r_end, Sp, Tp, st);
    }
}

/* bytes of pre-formed operands a product group may hold at once */
constexpr size_t kPrepackBudget = (size_t)4 << 30;

}  // namespace

int fmm_scale_c(int64_t m, int64_t n, double beta, double* C, int64_t ldc, cudaStream_t st)
{
    if (beta == 1.0 || m == 0 || n == 0) return FMM_OK;
    int64_t total = m * n;
    int blocks = (int)std::min<int64_t>((total + 255) / 256, 152 * 16);
    scale_c_kernel<<<blocks, 256, 0, st>>>(m, n, beta, C, ldc);
    fmm_count_launch(1);
    return cudaGetLastError() == cudaSuccess ? FMM_OK : FMM_ERR_CUDA;
}

/* Tile choice: the FP64 pipe is the bottleneck, so estimate each SM's FP64
 * work for every candidate (waves of CTAs over the SMs, two resident per SM,
 * times the FMAs per tile including the fused pack additions, over the
 * configuration's measured efficiency) and take the cheapest. Measured on
 * GB300 at m=n=k=16384: the 64-wide tiles with two CTAs per SM run classical
 * FP64 at 99% of the DFMA peak, the 128 x 128 tile with one CTA per SM
 * (248 registers) about 2% and FMM forms 5-14% slower, so it is not a
 * candidate; 32 x 32 serves grids too small to fill the SMs. */
int fmm_f64_launch(const AlgView& alg, int64_t m, int64_t n, int64_t k, double alpha,
                   const double* A, int64_t lda, const double* B, int64_t ldb,
                   double beta, double* C, int64_t ldc, cudaStream_t st)
{
    int rc = fmm_scale_c(m, n, beta, C, ldc, st);
    if (rc != FMM_OK) return rc;
    if (m == 0 || n == 0 || k == 0 || alpha == 0.0) return FMM_OK;
    if (alg.max_nnz_u > kMaxEntries || alg.max_nnz_v > kMaxEntries) return FMM_ERR_UNSUPPORTED;

    if (plain_classical(alg)) {
        const int ks = fmm_gpu_f64_sup_splits(m, n, k);
        if (ks >= 2) return sup_launch(m, n, k, alpha, A, lda, B, ldb, C, ldc, ks, st);
    }
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t me = (m + alg.mt - 1) / alg.mt, ne = (n + alg.nt - 1) / alg.nt, ke = (k + alg.kt - 1) / alg.kt;
    /* FMM algorithms form each product's operand combinations once, ahead of
     * the tiles (a stream-ordered temporary of at most kPrepackBudget per
     * product group), instead of once per tile position inside the kernel;
     * the values, and so the results, are the same either way. */
    const bool prepack = alg.R > 1;
    const double nu = prepack ? 1.0 : alg.avg_nnz_u, nv = prepack ? 1.0 : alg.avg_nnz_v;
    struct Cand { int id, bm, bn; double eff; };
    const Cand cands[4] = {{3, 64, 64, 1.0}, {4, 128, 64, 0.99}, {5, 64, 128, 0.99}, {2, 32, 32, 0.8}};
    double best = 0;
    int pick = 3;
    for (int c = 0; c < 4; ++c) {
        const int64_t bm = cands[c].bm, bn = cands[c].bn;
        const int64_t tiles = ((me + bm - 1) / bm) * ((ne + bn - 1) / bn);
        const double waves = (double)((tiles + 2 * (int64_t)sms - 1) / (2 * (int64_t)sms));
        const double work = (double)(bm * bn) * (1.0 + (nu - 1.0) / (double)bn + (nv - 1.0) / (double)bm +
                                                 4.0 / (double)bm);
        const double est = waves * work / cands[c].eff;
        if (c == 0 || est < best) { best = est; pick = cands[c].id; }
    }
    if (prepack) {
        const size_t per = (size_t)(me * ke + ke * ne) * sizeof(double);
        const int G = (int)std::max<size_t>(1, std::min<size_t>((size_t)alg.R, kPrepackBudget / std::max<size_t>(per, 1)));
        void* buf = nullptr;
        if (cudaMallocAsync(&buf, (size_t)G * per, st) == cudaSuccess) {
            double* Sbuf = (double*)buf;
            double* Tbuf = Sbuf + (size_t)G * me * ke;
            for (int r0 = 0; r0 < alg.R && rc == FMM_OK; r0 += G) {
                const int np = std::min(G, alg.R - r0);
                f64_combine_kernel<true><<<dim3((unsigned)(np * ((me + 255) / 256)), (unsigned)std::min<int64_t>(ke, 65535)),
                                           256, 0, st>>>(alg.tab, r0, np, A, lda, m, n, k, Sbuf);
                f64_combine_kernel<false><<<dim3((unsigned)(np * ((ke + 255) / 256)), (unsigned)std::min<int64_t>(ne, 65535)),
                                            256, 0, st>>>(alg.tab, r0, np, B, ldb, m, n, k, Tbuf);
                fmm_count_launch(2);
                rc = launch_pick(pick, alg, m, n, k, alpha, A, lda, B, ldb, C, ldc, r0, r0 + np, Sbuf, Tbuf, st);
            }
            if (cudaFreeAsync(buf, st) != cudaSuccess && rc == FMM_OK) rc = FMM_ERR_CUDA;
            return rc;
        }
        cudaGetLastError();   /* no temporary: the combinations stay fused into the kernel */
    }
    return launch_pick(pick, alg, m, n, k, alpha, A, lda, B, ldb, C, ldc, 0, alg.R, nullptr, nullptr, st);
}

/* Workspace of a batched FP64 launch: the work counter and the problem table. */
size_t fmm_f64_batch_ws_bytes(int count)
{
    return 256 + ((size_t)std::max(count, 0) * sizeof(F64Prob) + 255) / 256 * 256;
}

/* All problems of a batch in one persistent launch (plus the table-writer
 * launches and a counter reset). Problems are ordered by the FP64 work of one
 * of their items, largest first. Each result is identical to the problem
 * issued alone through fmm_f64_launch: every tile shape accumulates the
 * packed sums, the k loop and the products in the same order. */
namespace {
std::atomic<int> g_f64_batch_ctas{0};   /* 0: two CTAs per SM */
}  // namespace

extern "C" int fmm_gpu_set_f64_batch_ctas(int max_ctas)
{
    return g_f64_batch_ctas.exchange(max_ctas > 0 ? max_ctas : 0);
}

int fmm_f64_batch_launch(int count, const F64BatchItem* items, void* ws, size_t ws_bytes, cudaStream_t st)
{
    if (count <= 0) return FMM_OK;
    if (ws == nullptr || ws_bytes < fmm_f64_batch_ws_bytes(count)) return FMM_ERR_WORKSPACE;
    if (((uintptr_t)ws & 255) != 0) return FMM_ERR_ARG;
    std::vector<int> order;
    std::vector<double> cost(count, 0.0);
    for (int i = 0; i < count; ++i) {
        const F64BatchItem& it = items[i];
        if (it.alg.max_nnz_u > kMaxEntries || it.alg.max_nnz_v > kMaxEntries) return FMM_ERR_UNSUPPORTED;
        if (it.m == 0 || it.n == 0) continue;   /* nothing to do at all */
        if (it.k > 0 && it.alpha != 0.0 && plain_classical(it.alg)) {
            /* small/skinny classical problems take the same kernel as their
             * single calls (C := beta*C first, as there) */
            const int ks = fmm_gpu_f64_sup_splits(it.m, it.n, it.k);
            if (ks >= 2) {
                int rc = fmm_scale_c(it.m, it.n, it.beta, it.C, it.ldc, st);
                if (rc == FMM_OK) rc = sup_launch(it.m, it.n, it.k, it.alpha, it.A, it.lda, it.B, it.ldb, it.C,
                                                  it.ldc, ks, st);
                if (rc != FMM_OK) return rc;
                continue;
            }
        }
        const int64_t ke = (it.k + it.alg.kt - 1) / it.alg.kt;
        cost[i] = (it.k == 0 || it.alpha == 0.0) ? 1.0 : (double)it.alg.R * (double)(ke + 1);
        order.push_back(i);
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    std::vector<F64Prob> tab(order.size());
    int64_t items_total = 0;
    for (size_t q = 0; q < order.size(); ++q) {
        const F64BatchItem& it = items[order[q]];
        F64Prob& P = tab[q];
        P.tab = it.alg.tab;
        P.m = it.m; P.n = it.n; P.k = it.k;
        P.alpha = it.alpha; P.beta = it.beta;
        P.A = it.A; P.lda = it.lda; P.B = it.B; P.ldb = it.ldb; P.C = it.C; P.ldc = it.ldc;
        const int64_t me = (it.m + it.alg.mt - 1) / it.alg.mt, ne = (it.n + it.alg.nt - 1) / it.alg.nt;
        const int64_t tm = (me + kF64Bm - 1) / kF64Bm, tn = (ne + kF64Bn - 1) / kF64Bn;
        if (tm > 0x7fffffffLL || tn > 0x7fffffffLL) return FMM_ERR_UNSUPPORTED;
        P.tiles_m = (int)tm; P.tiles_n = (int)tn;
        P.item_begin = items_total;
        items_total += tm * tn;
    }
    if (tab.empty()) return FMM_OK;
    unsigned long long* counter = (unsigned long long*)ws;
    F64Prob* dtab = (F64Prob*)((uint8_t*)ws + 256);
    if (cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st) != cudaSuccess) return FMM_ERR_CUDA;
    for (size_t c0 = 0; c0 < tab.size(); c0 += kF64TableChunk) {
        F64TableChunk ch;
        ch.dst = dtab + c0;
        ch.count = (int)std::min<size_t>(kF64TableChunk, tab.size() - c0);
        memcpy(ch.p, tab.data() + c0, sizeof(F64Prob) * (size_t)ch.count);
        f64_table_write<<<1, 128, 0, st>>>(ch);
        fmm_count_launch(1);
    }
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t grid = std::min<int64_t>(items_total, 2 * (int64_t)sms);
    const int cap = g_f64_batch_ctas.load();
    if (cap > 0) grid = std::min<int64_t>(grid, cap);   /* items are drawn from a counter: any grid finishes them */
    if (g_f64_engine.load(std::memory_order_relaxed) == FMM_F64_MMA)
        fmm_f64_batch_kernel<true><<<(unsigned)grid, (kF64Bm / kF64Tm) * (kF64Bn / kF64Tn), 0, st>>>(
            dtab, (int)tab.size(), items_total, counter);
    else
        fmm_f64_batch_kernel<false><<<(unsigned)grid, (kF64Bm / kF64Tm) * (kF64Bn / kF64Tn), 0, st>>>(
            dtab, (int)tab.size(), items_total, counter);
    fmm_count_launch(1);
    return cudaGetLastError() == cudaSuccess ? FMM_OK : FMM_ERR_CUDA;
}

/* ---------------------------------------------------------------------------
 * Peak rates of the two FP64 paths of the SM, measured by compute-only
 * kernels (no memory traffic inside the loop): DFMA (fma.rn.f64, the plain
 * form's micro-kernel) and the FP64 tensor-core MMA (mma.sync m8n8k4 f64).
 * Each thread (DFMA) or warp (MMA) runs independent accumulation chains, so
 * the issue rate, not a dependency, bounds the loop.
 * ------------------------------------------------------------------------- */
namespace {

constexpr int kRateChains = 8;

/* NF DFMA chains per thread and NM FP64 MMA chains per warp, interleaved,
 * every chain with its own operand registers. On GB300 this compute-only loop
 * measures below what the DFMA GEMM kernel itself reaches (1.06 against
 * 1.25 TFLOP/s for the classical FP64 GEMM at 16384^3), so its figures are a
 * relative comparison of the two paths, not the pipe's peak. */
template <int NF, int NM>
__global__ void __launch_bounds__(256) fp64_rate_kernel(double* __restrict__ out, int iters)
{
    const int lane = threadIdx.x % 32;
    double a[kRateChains], bb[kRateChains], cc[kRateChains], d[kRateChains][2], x[kRateChains], y[kRateChains];
#pragma unroll
    for (int u = 0; u < kRateChains; ++u) {
        a[u] = 1e-3 * (threadIdx.x + u);
        bb[u] = 0.999999 - 1e-8 * u;
        cc[u] = 1e-9 * (u + 1);
        d[u][0] = 0.0;
        d[u][1] = 0.0;
        x[u] = 1e-3 * (lane + 1 + u);
        y[u] = 0.5 - 1e-3 * u;
    }
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < kRateChains; ++u) {
            if (u < NF) a[u] = fma(a[u], bb[u], cc[u]);
            if (u < NM)
                asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                             : "+d"(d[u][0]), "+d"(d[u][1])
                             : "d"(x[u]), "d"(y[u]));
        }
    }
    double sum = 0.0;
#pragma unroll
    for (int u = 0; u < kRateChains; ++u) sum += a[u] + d[u][0] + d[u][1];
    out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = sum;
}

}  // namespace

extern "C" int fmm_gpu_fp64_pipe_rates(double* dfma_tflops, double* dmma_tflops, double* mixed_tflops)
{
    if (dfma_tflops == nullptr || dmma_tflops == nullptr || mixed_tflops == nullptr) return FMM_ERR_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        return FMM_ERR_CUDA;
    const int blocks = 8 * sms, threads = 256, iters = 16384;
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * (size_t)blocks * threads) != cudaSuccess) return FMM_ERR_ALLOC;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc = FMM_OK;
    float ms[3] = {0.f, 0.f, 0.f};
    for (int which = 0; which < 3 && rc == FMM_OK; ++which) {
        for (int rep = 0; rep < 3; ++rep) {   /* the first launch warms up */
            cudaEventRecord(e0);
            if (which == 0) fp64_rate_kernel<kRateChains, 0><<<blocks, threads>>>(out, iters);
            else if (which == 1) fp64_rate_kernel<0, kRateChains><<<blocks, threads>>>(out, iters);
            else fp64_rate_kernel<kRateChains / 2, kRateChains / 2><<<blocks, threads>>>(out, iters);
            cudaEventRecord(e1);
            fmm_count_launch(1);
            if (cudaEventSynchronize(e1) != cudaSuccess || cudaGetLastError() != cudaSuccess) { rc = FMM_ERR_CUDA; break; }
            float t = 0.f;
            cudaEventElapsedTime(&t, e0, e1);
            if (rep > 0 && (ms[which] == 0.f || t < ms[which])) ms[which] = t;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (rc != FMM_OK) return rc;
    const double threads_total = (double)blocks * threads;
    const double fma_flops = threads_total * iters * 2.0, mma_flops = threads_total / 32.0 * iters * (2.0 * 8 * 8 * 4);
    *dfma_tflops = fma_flops * kRateChains / (ms[0] * 1e-3) / 1e12;
    *dmma_tflops = mma_flops * kRateChains / (ms[1] * 1e-3) / 1e12;
    *mixed_tflops = (fma_flops + mma_flops) * (kRateChains / 2) / (ms[2] * 1e-3) / 1e12;
    return FMM_OK;
}

extern "C" int fmm_gpu_set_f64_engine(int engine)
{
    if (engine != FMM_F64_DFMA && engine != FMM_F64_MMA) return -1;
    return g_f64_engine.exchange(engine);
}
