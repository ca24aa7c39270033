/*
 * fmm_gb300.h -- C ABI of the GB300 (sm_103a) fast-matrix-multiplication GEMM.
 *
 * The library computes C := beta*C + alpha*A*B for column-major FP64 matrices
 * with a one- or two-level <m~,k~,n~> fast matrix multiplication algorithm of
 * rank R, read from the reference's U/V/W coefficient files, in the "ABC"
 * form: the U- and V-weighted sums of A and B sub-blocks are formed while the
 * operand tiles are loaded, and each of the R products is added with its W
 * coefficients into every C sub-block it feeds.
 *
 * Reference interface each entry point replaces (paths inside fmm-blis):
 *   fmm_t, STRASSEN_FMM        plugin/bli_plugin_fmm_blis.h:58-68,
 *                              frame/base/bli_strassen_ab.c:12-24
 *   new_fmm / free_fmm         frame/include/bli_fmm.h:69-70,
 *                              frame/base/bli_read_fmm.c:24-86
 *   bl_clock                   frame/util/bli_fmm_util.c:106-109
 *   fmm_gpu_strassen_ab_ex     bli_strassen_ab_ex, frame/include/bli_fmm.h:74-81,
 *                              frame/base/bli_strassen_ab.c:123-295 (host buffers)
 *   fmm_gpu_strassen_ab        bli_strassen_ab, frame/include/bli_fmm.h:83-89,
 *                              frame/base/bli_strassen_ab.c:297-300
 *   fmm_gpu_dgemm              the device-resident form of bli_strassen_ab_ex
 *                              (the per-product loop at bli_strassen_ab.c:248-294
 *                              with the packm plugin kernel
 *                              plugin/ref_kernels/bli_packm_fmm_ref.c:51-148 and
 *                              the micro-kernel epilogue
 *                              plugin/ref_kernels/bli_gemm_fmm_ref.c:40-121)
 *   fmm_gpu_split_dgemm        the same GEMM computed from BF16 slices of the
 *                              packed FP64 combinations (split-precision form);
 *                              no counterpart function in the reference, whose
 *                              pack/epilogue plugin kernels it reuses in spirit
 *
 * Error behaviour: every fmm_gpu_* call returns an int status (FMM_OK = 0).
 * new_fmm keeps the reference's by-value signature; on a missing or malformed
 * file it returns an fmm_t with R == 0 and NULL arrays (the reference
 * dereferences NULL instead), and fmm_load returns the status.
 *
 * Layout: all matrices are column-major, element (i,j) at ptr[i + j*ld],
 * ld >= rows. Devices pointers are CUDA global memory of the current device.
 * `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 */
#ifndef FMM_GB300_H
#define FMM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- types -- */

/* Same field order and meaning as the reference's fmm_t
 * (plugin/bli_plugin_fmm_blis.h:58-68). U is (m_tilde*k_tilde) x R, V is
 * (k_tilde*n_tilde) x R, W is (m_tilde*n_tilde) x R, all row-major
 * (U[q*R + r]); row q of U is the A sub-block (q / k_tilde, q % k_tilde), row
 * q of V the B sub-block (q / n_tilde, q % n_tilde), row q of W the C
 * sub-block (q / n_tilde, q % n_tilde). */
typedef struct fmm_s {
    int m_tilde;
    int n_tilde;
    int k_tilde;
    int R;
    int* U;
    int* V;
    int* W;
} fmm_t;

enum fmm_status {
    FMM_OK = 0,
    FMM_ERR_ARG = 1,         /* bad dimension, stride, pointer or parameter */
    FMM_ERR_FILE = 2,        /* coefficient file cannot be opened */
    FMM_ERR_FORMAT = 3,      /* coefficient file malformed */
    FMM_ERR_ALLOC = 4,       /* host or device allocation failed */
    FMM_ERR_CUDA = 5,        /* a CUDA runtime/driver call failed */
    FMM_ERR_UNSUPPORTED = 6, /* size or option outside what the kernels handle */
    FMM_ERR_BRENT = 7,       /* coefficients do not satisfy the Brent equations */
    FMM_ERR_DEVICE = 8,      /* a kernel reported an error status (bounded wait expired) */
    FMM_ERR_WORKSPACE = 9,   /* caller workspace too small */
    FMM_ERR_SCRATCH = 10     /* problem larger than the static scratch of fmm_gpu_split_dgemm_noalloc */
};

/* ------------------------------------------------ coefficient algorithms -- */

/* Built-in Strassen <2,2,2>, R = 7, same coefficients as 222.txt
 * (frame/base/bli_strassen_ab.c:12-24). */
extern fmm_t STRASSEN_FMM;

/* Read a coefficient file (frame/base/bli_read_fmm.c:24-80). Header line
 * "m~ k~ n~ R" (the order the files are written in; the reference parses it
 * as m n k, which is only the same when k~ == n~), then m~k~ rows of U,
 * k~n~ rows of V and m~n~ rows of W; lines starting with '#' are skipped;
 * lines may be of any length. On failure returns R == 0, NULL arrays. */
fmm_t new_fmm(const char* file_name);

/* Free the arrays of an fmm_t from new_fmm/fmm_load/fmm_kron
 * (frame/base/bli_read_fmm.c:82-86). Never call it on STRASSEN_FMM. */
void free_fmm(fmm_t fmm);

/* Monotonic wall clock in seconds (frame/util/bli_fmm_util.c:106-109). */
double bl_clock(void);

/* new_fmm with a status code. */
int fmm_load(const char* file_name, fmm_t* out);

/* Check the Brent equations: for every A block (a,b), B block (b',c), C block
 * (a',c'), sum_r U*V*W == [a==a'][b==b'][c==c']. Returns FMM_OK or
 * FMM_ERR_BRENT; *n_bad (may be NULL) receives the number of violated
 * equations. */
int fmm_check_brent(const fmm_t* fmm, long* n_bad);

/* Two recursion levels as one flat algorithm: out = outer (x) inner with
 * m~ = m~o*m~i, k~ = k~o*k~i, n~ = n~o*n~i, R = Ro*Ri; sub-block (a,b) of the
 * flat grid is block (a % m~i, b % k~i) inside outer block (a / m~i, b / k~i).
 * out owns new arrays (free_fmm). */
int fmm_kron(const fmm_t* outer, const fmm_t* inner, fmm_t* out);

/* Deep copy (free_fmm the result). */
int fmm_copy(const fmm_t* src, fmm_t* dst);

/* Human-readable name of a status code. */
const char* fmm_status_string(int status);

/* ------------------------------------------------- GPU, plain FP64 form -- */

/* C := beta*C + alpha*A*B on the device, A m x k, B k x n, C m x n, FP64,
 * computed with `levels` recursion levels of `fmm` (levels == 0 or fmm ==
 * NULL: the classical FP64 GEMM kernel of this library). Sub-block sizes
 * follow the reference's split rule: along a dimension d split t ways the
 * first d % t blocks have ceil(d/t) elements and the rest floor(d/t); each
 * product is computed at the ceil size with zero fill. Asynchronous on
 * `stream`. */
int fmm_gpu_dgemm(const fmm_t* fmm, int levels,
                  int64_t m, int64_t n, int64_t k,
                  double alpha, const double* A, int64_t lda,
                  const double* B, int64_t ldb,
                  double beta, double* C, int64_t ldc,
                  void* stream);

/* Drop-in for bli_strassen_ab_ex with the obj_t operands unpacked into plain
 * HOST pointers, sizes and column strides (frame/base/bli_strassen_ab.c:123).
 * Copies A, B, C to the device, runs fmm_gpu_dgemm with one level of `fmm`,
 * copies C back, synchronously. */
int fmm_gpu_strassen_ab_ex(double alpha, const double* A, int64_t lda,
                           const double* B, int64_t ldb,
                           double beta, double* C, int64_t ldc,
                           int64_t m, int64_t n, int64_t k,
                           fmm_t fmm);

/* fmm_gpu_strassen_ab_ex for operands with any layout, the way a BLIS obj_t
 * describes them (frame/base/bli_strassen_ab.c:143-149 reads its operands
 * through obj_t accessors): element (i, j) of X at X[i*rs_x + j*cs_x], all
 * strides >= 1. Row-major operands and transposed ones (a transposed
 * column-major operand is a row-major one of the transposed shape) take one
 * pitched copy and a transpose on the device; other strides are gathered on
 * the host. Only C's own elements are written back. The result equals the
 * column-major call's bit for bit. */
int fmm_gpu_strassen_ab_gen(double alpha, const double* A, int64_t rs_a, int64_t cs_a,
                            const double* B, int64_t rs_b, int64_t cs_b,
                            double beta, double* C, int64_t rs_c, int64_t cs_c,
                            int64_t m, int64_t n, int64_t k, fmm_t fmm);

/* Drop-in for bli_strassen_ab (frame/base/bli_strassen_ab.c:297-300):
 * fmm_gpu_strassen_ab_ex with STRASSEN_FMM. */
int fmm_gpu_strassen_ab(double alpha, const double* A, int64_t lda,
                        const double* B, int64_t ldb,
                        double beta, double* C, int64_t ldc,
                        int64_t m, int64_t n, int64_t k);

/* ------------------------------------ GPU, split-precision (Ozaki) form -- */

/* Bytes of device workspace recommended for fmm_gpu_split_dgemm: products
 * are processed in groups (all products of a group are packed, multiplied and
 * added into C in one pass), and this size holds the largest group that fits
 * in 32 GiB; when that is all R products, it holds two groups of ceil(R/2)
 * instead, whose packs and C updates overlap the other group's GEMM. Any
 * smaller workspace that holds one product's digit slices and level
 * accumulators also works, with smaller groups; the result is the same bit
 * for bit whatever the grouping. */
size_t fmm_gpu_split_workspace_size(const fmm_t* fmm, int levels,
                                    int64_t m, int64_t n, int64_t k,
                                    int slices);

/* C := beta*C + alpha*A*B computed as the FMM above, but each product's FP64
 * operand combinations are split (after a power-of-two row/column scaling)
 * into `slices` BF16 digit slices of 8 bits; all slice pairs (s,t) with
 * s + t <= slices + 1 are multiplied on the tcgen05 tensor cores with exact
 * integer-valued FP32 accumulation, and recombined in FP64. slices in 2..8.
 * `workspace` (256-byte aligned) holds at least one product's slices and
 * level accumulators; fmm_gpu_split_workspace_size gives the recommended
 * size. Asynchronous on `stream`. */
int fmm_gpu_split_dgemm(const fmm_t* fmm, int levels,
                        int64_t m, int64_t n, int64_t k,
                        double alpha, const double* A, int64_t lda,
                        const double* B, int64_t ldb,
                        double beta, double* C, int64_t ldc,
                        int slices, void* workspace, size_t workspace_bytes,
                        void* stream);

/* Slice formats of the split form. No counterpart in the reference. */
#define FMM_SPLIT_BF16 0      /* base-256 digits as BF16, tcgen05 kind::f16, slices 2..8 */
#define FMM_SPLIT_FP8_E4M3 1  /* base-32 digits as FP8-E4M3, tcgen05 kind::f8f6f4, slices 2..12 */

/* fmm_gpu_split_workspace_size for a slice format (FMM_SPLIT_*). */
size_t fmm_gpu_split_workspace_size_fmt(const fmm_t* fmm, int levels,
                                        int64_t m, int64_t n, int64_t k,
                                        int slices, int format);

/* fmm_gpu_split_dgemm with a slice format: FMM_SPLIT_BF16 (identical to
 * fmm_gpu_split_dgemm) or FMM_SPLIT_FP8_E4M3: 5-bit digits in [-16, 16]
 * stored as FP8-E4M3, multiplied at the FP8 tensor rate with the same
 * per-row/per-column power-of-two scales and exact integer accumulation, so
 * each slice carries 5 bits instead of 8. No counterpart in the reference. */
int fmm_gpu_split_dgemm_fmt(const fmm_t* fmm, int levels,
                            int64_t m, int64_t n, int64_t k,
                            double alpha, const double* A, int64_t lda,
                            const double* B, int64_t ldb,
                            double beta, double* C, int64_t ldc,
                            int slices, int format, void* workspace, size_t workspace_bytes,
                            void* stream);

/* The split form on HOST buffers: bli_strassen_ab_ex's operands (column-major
 * host pointers with leading dimensions, as fmm_gpu_strassen_ab_ex takes
 * them) multiplied in the split-precision form with `levels` levels of `fmm`
 * (0: classical), `slices` digit slices of `format` (FMM_SPLIT_*).
 * Synchronous: returns when C holds the result. The copies overlap the
 * device work: B and C travel while A's slices are formed and under the
 * GEMM. Pinned host memory copies fastest; pageable memory works too. The
 * device copies and the workspace are kept between calls (grow-only, per
 * device) until fmm_gpu_release_host_buffers. The result equals
 * fmm_gpu_split_dgemm_fmt's on the same values bit for bit. No counterpart
 * in the reference. */
int fmm_gpu_split_strassen_ab_ex(double alpha, const double* A, int64_t lda,
                                 const double* B, int64_t ldb,
                                 double beta, double* C, int64_t ldc,
                                 int64_t m, int64_t n, int64_t k,
                                 fmm_t fmm, int levels, int slices, int format);

/* fmm_gpu_split_strassen_ab_ex for operands of any layout, as
 * fmm_gpu_strassen_ab_gen takes them (element (i, j) of X at
 * X[i*rs_x + j*cs_x], all strides >= 1): column-major operands go through the
 * overlapped host-buffer call, others are made column-major on the device,
 * multiplied and C written back in place (only C's own elements). The result
 * equals the column-major call's bit for bit. No counterpart in the
 * reference. */
int fmm_gpu_split_strassen_ab_gen(double alpha, const double* A, int64_t rs_a, int64_t cs_a,
                                  const double* B, int64_t rs_b, int64_t cs_b,
                                  double beta, double* C, int64_t rs_c, int64_t cs_c,
                                  int64_t m, int64_t n, int64_t k,
                                  fmm_t fmm, int levels, int slices, int format);

/* Frees the current device's buffers kept by fmm_gpu_split_strassen_ab_ex. */
void fmm_gpu_release_host_buffers(void);

/* Pinned host memory for the operands of the host-buffer entry points:
 * `bytes` of zeroed memory on transparent huge pages where the host offers
 * them (buffers of at least one huge page), page-locked for the GPU. The copy
 * engines translate fewer, larger pages, so copies keep the host link's rate
 * even when they start after the host has been idle (measured on a GB300
 * host, 2 GiB after 5 s idle: 10.2 ms from huge pages, 13.7 ms from
 * cudaHostAlloc memory, 40.5 ms from registered 64 KiB pages). Release with
 * fmm_gpu_host_free. Needs a GPU (FMM_ERR_CUDA without one). No counterpart
 * in the reference (whose operands are BLIS objects in host memory). */
int fmm_gpu_host_alloc(size_t bytes, void** ptr);
int fmm_gpu_host_free(void* ptr);

/* Timeline of fmm_gpu_split_strassen_ab_ex calls, while enabled: CUDA events
 * recorded inside the call. fmm_gpu_read_host_timeline fills ms[0..5] for the
 * last call: device milliseconds from the start of A's upload to A on the
 * device, B on the device, the first GEMM launch's start, the last GEMM
 * launch's end and C's last column chunk back on the host, then the call's
 * host wall time. Returns how many values it wrote. Recorded when the call
 * takes its overlapped path (all products' C updates in the element-major
 * form). No counterpart in the reference. */
void fmm_gpu_set_host_timeline(int enable);
int fmm_gpu_read_host_timeline(double* ms, int count);

/* ------------------------------------------------------- GPU, batched -- */

/* One GEMM of a batch: C := beta*C + alpha*A*B with `levels` levels of `fmm`
 * (NULL: classical), in the split form with `slices` digit slices of
 * `format` (FMM_SPLIT_*), or in the plain FP64 form when slices == 0. Device
 * pointers, column-major. */
typedef struct fmm_batch_problem_s {
    const fmm_t* fmm;
    int levels;
    int slices;
    int64_t m, n, k;
    double alpha;
    const double* A;
    int64_t lda;
    const double* B;
    int64_t ldb;
    double beta;
    double* C;
    int64_t ldc;
    int format;
} fmm_batch_problem;

/* Recommended workspace for fmm_gpu_batch_dgemm (capped at 32 GiB; any size
 * that holds the largest problem's one-product workspace works). */
size_t fmm_gpu_batch_workspace_size(int count, const fmm_batch_problem* problems);

/* Runs `count` independent GEMMs (their C regions must not overlap). Plain
 * FP64 problems run in one persistent launch over all their (problem, tile
 * position) work items. Split-form problems go in waves of up to 80 whose
 * workspaces fit together: every problem of a wave is packed, one persistent
 * tensor-core launch covers all their (problem, product, tile) work items,
 * then each C is updated. Each result is bit-identical to the problem's own
 * single call. No counterpart in the reference (which runs one GEMM per
 * call). Asynchronous on `stream`. */
int fmm_gpu_batch_dgemm(int count, const fmm_batch_problem* problems,
                        void* workspace, size_t workspace_bytes, void* stream);

/* fmm_gpu_split_dgemm for callers that must not allocate device memory
 * while they run: a plug-in working in memory a host application hands it
 * (the application's own caching allocator owns the device, and a cudaMalloc
 * behind its back can fail or fragment its pool), a process whose device
 * memory is fully reserved, a latency-bound loop that cannot afford
 * cudaFree's implicit device synchronization. It calls no cudaMalloc, cudaFree or other device
 * allocator. No counterpart in the reference. The algorithm table and the
 * workspace live in one static device array of 64 MiB that every GPU loading
 * the library keeps until exit; a problem whose workspace (slices and level
 * accumulators for at least one product) does not fit returns
 * FMM_ERR_SCRATCH. The table is written by kernels that carry it as their
 * launch parameter, so no host buffer outlives the call. The first call on a
 * device looks up the array's device address and keeps it for the process;
 * make that first call before any stream capture, and do not use the entry
 * point after cudaDeviceReset on that device. All calls share the array and
 * each call rewrites what it uses, so calls whose GPU work overlaps (other
 * streams, other threads) race: serialize them. */
int fmm_gpu_split_dgemm_noalloc(const fmm_t* fmm, int levels,
                                int64_t m, int64_t n, int64_t k,
                                double alpha, const double* A, int64_t lda,
                                const double* B, int64_t ldb,
                                double beta, double* C, int64_t ldc,
                                int slices, void* stream);

/* Per-launch timing of the split form's tensor-core GEMM kernel: while
 * enabled, a CUDA event pair is recorded on the launch stream around each
 * launch; fmm_gpu_read_kernel_timing waits for them and returns the summed
 * milliseconds, the launch count and the number of FMM products those
 * launches computed (one launch covers a group of products) since the last
 * read. */
void fmm_gpu_set_kernel_timing(int enable);
int fmm_gpu_read_kernel_timing(double* total_ms, uint64_t* launches, uint64_t* products);

/* Upper bound on the CTAs of the persistent FP64 batch launch of
 * fmm_gpu_batch_dgemm (0, the default: two per SM). Its work items are drawn
 * from a counter, so any grid finishes them; a small cap leaves the other SMs
 * free for work on other streams (a server keeps split-form requests flowing
 * beside long FP64 batches this way). Results do not depend on it. Returns
 * the previous value. No counterpart in the reference. */
int fmm_gpu_set_f64_batch_ctas(int max_ctas);

/* Smallest per-product row count m_e = ceil(m / m~^levels) from which the
 * split form's GEMM runs on CTA pairs (clusters of two SMs, 256 x 256 tiles,
 * tcgen05.mma cta_group::2) instead of one SM per 128 x 256 tile; applies to
 * single and batched calls. Default 1024, values below 1024 are raised to it,
 * INT_MAX keeps every problem on single-SM tiles. Results are bit-identical
 * either way (every tile's sums are exact); only the speed differs. Returns
 * the previous value. No counterpart in the reference. */
int fmm_gpu_set_split_pair_rows(int min_rows);

/* Micro-kernel of the plain FP64 form, for single and batched calls alike:
 * FMM_F64_DFMA (register-blocked fma.rn.f64) or FMM_F64_MMA (the FP64
 * tensor-core path, mma.sync m8n8k4 f64, fragments from the same fused-pack
 * tiles). Both accumulate every C element over k in increasing order; on
 * GB300 they share one FP64 pipe (fmm_gpu_fp64_pipe_rates). Returns the
 * previous engine, or -1 for an unknown one. No counterpart in the reference
 * (whose micro-kernel is the haswell dgemm assembly kernel). */
enum fmm_f64_engine { FMM_F64_DFMA = 0, FMM_F64_MMA = 1 };
int fmm_gpu_set_f64_engine(int engine);

/* The small/skinny classical path of the plain FP64 form, the counterpart of
 * BLIS's "sup" kernels for small and skinny shapes (blis/kernels/haswell/3/
 * sup): a classical FP64 GEMM (levels 0) whose output has at most 128 tiles
 * of 32 x 32 and whose k is long runs as clusters of CTAs that split k into
 * 2..8 chunks of at least 256 and add the chunks' partial tiles through
 * distributed shared memory in chunk order, instead of one CTA per tile down
 * all of k. Returns the number of chunks for an m x n x k problem (0: the
 * regular kernel). It depends on the shape only, so single and batched calls
 * of a problem give the same bits; it needs no GPU. */
int fmm_gpu_f64_sup_splits(int64_t m, int64_t n, int64_t k);

/* Rates (TFLOP/s) of the GPU's two FP64 paths from compute-only kernels
 * with independent chains over every SM, timed with CUDA events (best of two
 * launches after a warm-up): DFMA (fma.rn.f64, which the plain form's
 * micro-kernel uses), the FP64 tensor-core MMA (mma.sync m8n8k4 f64), and
 * both interleaved in one kernel (their sum; about the larger alone when they
 * share one pipe). On GB300 these loops stay below the rate the DFMA GEMM
 * reaches, so they compare the paths rather than give the pipe's peak. A
 * measurement utility; no counterpart in the reference. */
int fmm_gpu_fp64_pipe_rates(double* dfma_tflops, double* dmma_tflops, double* mixed_tflops);

/* Number of kernels the library launched since load (all entry points). */
uint64_t fmm_gpu_launch_count(void);

/* Last device-side error word (0 = none) recorded by a kernel whose bounded
 * wait expired; reading it synchronizes the device. Clears it. */
int fmm_gpu_take_device_error(void);

/* Self-test of the kernels' failure path: one CTA of 64 threads waits, with
 * the bounded mbarrier wait the GEMM kernels use, on a barrier nothing
 * arrives at. The wait gives up after its limit (2 s), records an error code
 * in the device error word, makes the other threads give up too, and the
 * kernel ends; the call then reads the word as the synchronous entry points
 * do. Returns FMM_ERR_DEVICE (word cleared) when the failure path worked,
 * *threads_gave_up = 64. No counterpart in the reference. */
int fmm_gpu_selftest_wait_expiry(int* threads_gave_up);

#ifdef __cplusplus
}
#endif

#endif /* FMM_GB300_H */
