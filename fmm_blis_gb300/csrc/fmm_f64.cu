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

#include <algorithm>

namespace {

constexpr int kMaxEntries = 256;  /* nonzero coefficients per product column */

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

template <int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
fmm_f64_kernel(const int* __restrict__ tab, int64_t m, int64_t n, int64_t k,
               double alpha, const double* __restrict__ A, int64_t lda,
               const double* __restrict__ B, int64_t ldb,
               double* __restrict__ C, int64_t ldc, int tiles_m)
{
    constexpr int NT = (BM / TM) * (BN / TN);
    constexpr int RT = BM / TM;  /* thread rows */
    constexpr int CT = BN / TN;  /* thread cols */
    static_assert(NT % BM == 0 && NT % BK == 0, "tile/thread mapping");

    __shared__ double As[BK][BM + 1];
    __shared__ double Bs[BK][BN + 1];
    __shared__ Entry ue[kMaxEntries];
    __shared__ Entry ve[kMaxEntries];

    const int mt = tab[0], kt = tab[1], nt = tab[2], R = tab[3];
    const int* u_off = tab + FMM_ALG_HDR;
    const int* v_off = u_off + (R + 1);
    const int* w_off = v_off + (R + 1);
    const int* ents = w_off + (R + 1);          /* (part, coef) pairs */
    const int* u_ent = ents;
    const int* v_ent = ents + 2 * u_off[R];
    const int* w_ent = v_ent + 2 * v_off[R];

    const int64_t me = (m + mt - 1) / mt, ne = (n + nt - 1) / nt, ke = (k + kt - 1) / kt;
    const int ti = blockIdx.x % tiles_m, tj = blockIdx.x / tiles_m;
    const int64_t i0 = (int64_t)ti * BM, j0 = (int64_t)tj * BN;
    const int tid = threadIdx.x;
    const int tr = tid % RT, tc = tid / RT;

    for (int r = 0; r < R; ++r) {
        const int wb = w_off[r], we = w_off[r + 1];
        if (wb == we) continue;
        const int ub = u_off[r], ue_n = u_off[r + 1] - ub;
        const int vb = v_off[r], ve_n = v_off[r + 1] - vb;
        __syncthreads();  /* previous product finished with ue/ve */
        stage_entries(u_ent, ub, ub + ue_n, kt, mt, A, lda, m, k, ue);
        stage_entries(v_ent, vb, vb + ve_n, nt, kt, B, ldb, k, n, ve);
        __syncthreads();

        double acc[TM][TN];
#pragma unroll
        for (int a = 0; a < TM; ++a)
#pragma unroll
            for (int b = 0; b < TN; ++b) acc[a][b] = 0.0;

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
                for (int t = 0; t < NA; ++t) As[tid / BM + t * (NT / BM)][li] = s[t];
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
                for (int t = 0; t < NB; ++t) Bs[lp][tid / BK + t * (NT / BK)] = s[t];
            }
            __syncthreads();
#pragma unroll 4
            for (int kk = 0; kk < BK; ++kk) {
                double a[TM], b[TN];
#pragma unroll
                for (int x = 0; x < TM; ++x) a[x] = As[kk][tr + x * RT];
#pragma unroll
                for (int y = 0; y < TN; ++y) b[y] = Bs[kk][tc + y * CT];
#pragma unroll
                for (int x = 0; x < TM; ++x)
#pragma unroll
                    for (int y = 0; y < TN; ++y) acc[x][y] = fma(a[x], b[y], acc[x][y]);
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
#pragma unroll
            for (int y = 0; y < TN; ++y) {
                const int64_t gj = j0 + tc + y * CT;
                if (gj >= cl) continue;
#pragma unroll
                for (int x = 0; x < TM; ++x) {
                    const int64_t gi = i0 + tr + x * RT;
                    if (gi < rl) {
                        double* p = cb + gi + gj * ldc;
                        *p = fma(lam, acc[x][y], *p);
                    }
                }
            }
        }
    }
    (void)me; (void)ne;
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

template <int BM, int BN, int BK, int TM, int TN>
int launch_cfg(const AlgView& alg, int64_t m, int64_t n, int64_t k, double alpha,
               const double* A, int64_t lda, const double* B, int64_t ldb, double* C,
               int64_t ldc, cudaStream_t st)
{
    const int64_t me = (m + alg.mt - 1) / alg.mt, ne = (n + alg.nt - 1) / alg.nt;
    const int64_t tm = (me + BM - 1) / BM, tn = (ne + BN - 1) / BN;
    if (tm * tn > 0x7fffffffLL) return FMM_ERR_UNSUPPORTED;
    fmm_f64_kernel<BM, BN, BK, TM, TN><<<(unsigned)(tm * tn), (BM / TM) * (BN / TN), 0, st>>>(
        alg.tab, m, n, k, alpha, A, lda, B, ldb, C, ldc, (int)tm);
    fmm_count_launch(1);
    return cudaGetLastError() == cudaSuccess ? FMM_OK : FMM_ERR_CUDA;
}

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

    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t me = (m + alg.mt - 1) / alg.mt, ne = (n + alg.nt - 1) / alg.nt;
    struct Cand { int id, bm, bn; double eff; };
    const Cand cands[4] = {{3, 64, 64, 1.0}, {4, 128, 64, 0.99}, {5, 64, 128, 0.99}, {2, 32, 32, 0.8}};
    double best = 0;
    int pick = 3;
    for (int c = 0; c < 4; ++c) {
        const int64_t bm = cands[c].bm, bn = cands[c].bn;
        const int64_t tiles = ((me + bm - 1) / bm) * ((ne + bn - 1) / bn);
        const double waves = (double)((tiles + 2 * (int64_t)sms - 1) / (2 * (int64_t)sms));
        const double work = (double)(bm * bn) * (1.0 + (alg.avg_nnz_u - 1.0) / (double)bn +
                                                 (alg.avg_nnz_v - 1.0) / (double)bm + 4.0 / (double)bm);
        const double est = waves * work / cands[c].eff;
        if (c == 0 || est < best) { best = est; pick = cands[c].id; }
    }
    switch (pick) {
    case 3: return launch_cfg<64, 64, 32, 4, 4>(alg, m, n, k, alpha, A, lda, B, ldb, C, ldc, st);
    case 4: return launch_cfg<128, 64, 16, 8, 4>(alg, m, n, k, alpha, A, lda, B, ldb, C, ldc, st);
    case 5: return launch_cfg<64, 128, 16, 4, 8>(alg, m, n, k, alpha, A, lda, B, ldb, C, ldc, st);
    default: return launch_cfg<32, 32, 32, 2, 2>(alg, m, n, k, alpha, A, lda, B, ldb, C, ldc, st);
    }
}
