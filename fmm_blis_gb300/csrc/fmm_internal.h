/*
 * Internal declarations shared by the CUDA translation units.
 *
 * An FMM algorithm reaches the kernels as a flat int32 table ("alg table"),
 * uploaded once per distinct algorithm and cached on each device:
 *
 *   [0] mt  [1] kt  [2] nt  [3] R
 *   [4 .. 4+R]           u_off : start of product r's U entries (R+1 values)
 *   [.. +R+1]            v_off
 *   [.. +R+1]            w_off
 *   then U entries (part, coef) pairs, V entries, W entries,
 *   then wp_off (m~n~ + 1 values) and the W entries grouped by C sub-block,
 *   (product, coef) pairs in increasing product order.
 *
 * Only nonzero coefficients are stored, in increasing part order, so the
 * kernels add the A (B) sub-blocks in the same order as the reference's pack
 * kernel (plugin/ref_kernels/bli_packm_fmm_ref.c:122-147) and skip its 0*x
 * additions.
 */
#ifndef FMM_INTERNAL_H
#define FMM_INTERNAL_H

#include <stdint.h>
#include <cuda_runtime.h>
#include <vector>
#include "../../include/fmm_gb300.h"

#define FMM_ALG_HDR 4

struct AlgView {
    const int* tab;  /* device pointer to the table */
    const int* htab; /* host copy of the same table */
    int mt, kt, nt, R;
    int max_nnz_u, max_nnz_v, max_nnz_w;
    double avg_nnz_u, avg_nnz_v, avg_nnz_w;
    int tab_len;
};

/* Sub-block geometry along a dimension of length d split t ways, block i
 * (frame/base/bli_strassen_ab.c:86-121): the first d % t blocks have one
 * extra element. */
__host__ __device__ __forceinline__ void fmm_part_geom(int64_t d, int t, int i,
                                                       int64_t* off, int64_t* len)
{
    int64_t base = d / t, rem = d % t;
    *off = (int64_t)i * base + (i < rem ? (int64_t)i : rem);
    *len = base + (i < rem ? 1 : 0);
}

/* 32-bit form for device code (sizes below 2^31), avoiding 64-bit division. */
__host__ __device__ __forceinline__ void fmm_part_geom32(int d, int t, int i, int* off, int* len)
{
    const int base = d / t, rem = d - base * t;
    *off = i * base + (i < rem ? i : rem);
    *len = base + (i < rem ? 1 : 0);
}

/* Host helpers implemented in fmm_api.cu */
int fmm_flatten(const fmm_t* fmm, int levels, fmm_t* flat, int* owned);
int fmm_alg_get(const fmm_t* flat, AlgView* out);  /* upload/cache */
/* host table and view without any device allocation (view.tab left NULL) */
int fmm_alg_describe(const fmm_t* flat, std::vector<int>* table, AlgView* out);
void fmm_count_launch(uint64_t n);
int* fmm_device_error_word(void);                 /* device pointer */
int fmm_device_error_status(void);                /* FMM_ERR_DEVICE if a wait expired (clears it), else FMM_OK */

/* FP64 form (fmm_f64.cu) */
int fmm_f64_launch(const AlgView& alg, int64_t m, int64_t n, int64_t k,
                   double alpha, const double* A, int64_t lda,
                   const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
                   cudaStream_t st);

/* batched FP64 form (fmm_f64.cu): one persistent launch over every
 * (problem, tile position) item */
struct F64BatchItem {
    AlgView alg;
    int64_t m, n, k;
    double alpha, beta;
    const double* A;
    int64_t lda;
    const double* B;
    int64_t ldb;
    double* C;
    int64_t ldc;
};
size_t fmm_f64_batch_ws_bytes(int count);
int fmm_f64_batch_launch(int count, const F64BatchItem* items, void* ws, size_t ws_bytes, cudaStream_t st);

/* split form (fmm_split.cu) */
/* fmt: 0 = BF16 slices, 1 = FP8-E4M3 slices */
size_t fmm_split_ws_bytes(const AlgView& alg, int64_t m, int64_t n, int64_t k, int slices, int fmt);
/* split form on host buffers, copies overlapped with the device work */
int fmm_split_host(const AlgView& alg, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
                   int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc, int s, int fmt);
void fmm_split_host_release();
int fmm_split_launch(const AlgView& alg, int64_t m, int64_t n, int64_t k,
                     double alpha, const double* A, int64_t lda,
                     const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
                     int slices, int fmt, void* ws, size_t ws_bytes, cudaStream_t st);

/* Reads one byte of every page of the host memory [p, p + bytes) on the
 * calling thread. On GB300 hosts a copy engine reading or writing pinned
 * host memory whose pages the host has not touched for a few seconds ran at a
 * fraction of the link rate (2 GiB in 33.7 ms instead of 10.2 ms); touching
 * one byte per page first (about 1 ms for 2 GiB of 64 KiB pages) restored
 * the full rate. */
void fmm_touch_host(const void* p, size_t bytes);

/* Pitched copy of `height` rows of `width` bytes between host and device.
 * When both pitches equal the width the rows are one contiguous block and go
 * as a single linear copy (cudaMemcpyAsync); otherwise as a pitched copy. The
 * host side's pages are touched first (fmm_touch_host). */
inline cudaError_t fmm_copy2d_async(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width,
                                    size_t height, cudaMemcpyKind kind, cudaStream_t st)
{
    if (width == 0 || height == 0) return cudaSuccess;
    if (kind == cudaMemcpyHostToDevice) fmm_touch_host(src, (height - 1) * spitch + width);
    if (kind == cudaMemcpyDeviceToHost) fmm_touch_host(dst, (height - 1) * dpitch + width);
    if (dpitch == width && spitch == width) return cudaMemcpyAsync(dst, src, width * height, kind, st);
    return cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, height, kind, st);
}

/* C := beta*C (fmm_f64.cu) */
int fmm_scale_c(int64_t m, int64_t n, double beta, double* C, int64_t ldc, cudaStream_t st);

#endif
