/*
 * C ABI entry points (include/fmm_gb300.h): argument checks, flattening of
 * multi-level algorithms, the per-device cache of algorithm tables, and the
 * host-buffer drop-in for bli_strassen_ab_ex (frame/base/bli_strassen_ab.c:123).
 */
#include "fmm_internal.h"

#include <sys/mman.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

namespace {

std::atomic<uint64_t> g_launches{0};

__device__ int g_device_error;

struct CachedAlg {
    int device;
    std::vector<int> table;
    int* dtab;
    AlgView view;
};

std::mutex g_mu;
std::vector<CachedAlg*> g_cache;

int* g_err_ptr[64];
bool g_err_init[64];

bool ld_ok(int64_t ld, int64_t rows) { return ld >= (rows > 1 ? rows : 1); }

std::vector<int> build_table(const fmm_t* f)
{
    const int R = f->R;
    const int a = f->m_tilde * f->k_tilde, b = f->k_tilde * f->n_tilde, c = f->m_tilde * f->n_tilde;
    std::vector<int> off_u(R + 1), off_v(R + 1), off_w(R + 1);
    std::vector<int> eu, ev, ew;
    for (int r = 0; r < R; ++r) {
        off_u[r] = (int)eu.size() / 2;
        for (int q = 0; q < a; ++q)
            if (int x = f->U[(size_t)q * R + r]) { eu.push_back(q); eu.push_back(x); }
        off_v[r] = (int)ev.size() / 2;
        for (int q = 0; q < b; ++q)
            if (int x = f->V[(size_t)q * R + r]) { ev.push_back(q); ev.push_back(x); }
        off_w[r] = (int)ew.size() / 2;
        for (int q = 0; q < c; ++q)
            if (int x = f->W[(size_t)q * R + r]) { ew.push_back(q); ew.push_back(x); }
    }
    off_u[R] = (int)eu.size() / 2;
    off_v[R] = (int)ev.size() / 2;
    off_w[R] = (int)ew.size() / 2;
    std::vector<int> t;
    t.push_back(f->m_tilde); t.push_back(f->k_tilde); t.push_back(f->n_tilde); t.push_back(R);
    t.insert(t.end(), off_u.begin(), off_u.end());
    t.insert(t.end(), off_v.begin(), off_v.end());
    t.insert(t.end(), off_w.begin(), off_w.end());
    t.insert(t.end(), eu.begin(), eu.end());
    t.insert(t.end(), ev.begin(), ev.end());
    t.insert(t.end(), ew.begin(), ew.end());
    /* W by C sub-block: for each part p, its (product, coef) entries in
     * increasing product order */
    std::vector<int> off_p(c + 1), ep;
    for (int q = 0; q < c; ++q) {
        off_p[q] = (int)ep.size() / 2;
        for (int r = 0; r < R; ++r)
            if (int x = f->W[(size_t)q * R + r]) { ep.push_back(r); ep.push_back(x); }
    }
    off_p[c] = (int)ep.size() / 2;
    t.insert(t.end(), off_p.begin(), off_p.end());
    t.insert(t.end(), ep.begin(), ep.end());
    return t;
}

AlgView view_of(const std::vector<int>& table, const int* dtab)
{
    const int* t = table.data();
    AlgView v;
    v.tab = dtab;
    v.htab = t;
    v.mt = t[0]; v.kt = t[1]; v.nt = t[2]; v.R = t[3];
    const int* ou = t + FMM_ALG_HDR;
    const int* ov = ou + v.R + 1;
    const int* ow = ov + v.R + 1;
    v.max_nnz_u = v.max_nnz_v = v.max_nnz_w = 0;
    for (int r = 0; r < v.R; ++r) {
        v.max_nnz_u = std::max(v.max_nnz_u, ou[r + 1] - ou[r]);
        v.max_nnz_v = std::max(v.max_nnz_v, ov[r + 1] - ov[r]);
        v.max_nnz_w = std::max(v.max_nnz_w, ow[r + 1] - ow[r]);
    }
    v.avg_nnz_u = (double)ou[v.R] / v.R;
    v.avg_nnz_v = (double)ov[v.R] / v.R;
    v.avg_nnz_w = (double)ow[v.R] / v.R;
    v.tab_len = (int)table.size();
    return v;
}

void fill_view(CachedAlg* c) { c->view = view_of(c->table, c->dtab); }

bool valid_fmm(const fmm_t* f)
{
    return f && f->R > 0 && f->m_tilde > 0 && f->k_tilde > 0 && f->n_tilde > 0 && f->U && f->V && f->W;
}

}  // namespace

void fmm_count_launch(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

extern "C" uint64_t fmm_gpu_launch_count(void) { return g_launches.load(); }

int* fmm_device_error_word(void)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_err_init[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_device_error) != cudaSuccess) return nullptr;
        g_err_ptr[dev] = (int*)p;
        g_err_init[dev] = true;
    }
    return g_err_ptr[dev];
}

/* FMM_ERR_DEVICE (and the word cleared) when a kernel recorded an expired
 * wait, else FMM_OK; for synchronous calls, after their work has finished. */
int fmm_device_error_status(void)
{
    int v = 0, zero = 0;
    if (cudaMemcpyFromSymbol(&v, g_device_error, sizeof(int)) != cudaSuccess) return FMM_ERR_CUDA;
    if (v == 0) return FMM_OK;
    cudaMemcpyToSymbol(g_device_error, &zero, sizeof(int));
    return FMM_ERR_DEVICE;
}

extern "C" int fmm_gpu_take_device_error(void)
{
    int v = 0, zero = 0;
    if (cudaDeviceSynchronize() != cudaSuccess) return -1;
    if (cudaMemcpyFromSymbol(&v, g_device_error, sizeof(int)) != cudaSuccess) return -1;
    if (v != 0) cudaMemcpyToSymbol(g_device_error, &zero, sizeof(int));
    return v;
}

namespace {
std::mutex g_brent_mu;
std::vector<std::vector<int>> g_brent_ok;   /* algorithms already verified, serialized */
}  // namespace

/* The Brent check, once per distinct algorithm of the process (a flat
 * two-level algorithm has up to 16.7 M equations; calls reuse the result). */
static int brent_checked(const fmm_t* f)
{
    const size_t a = (size_t)f->m_tilde * f->k_tilde * f->R, b = (size_t)f->k_tilde * f->n_tilde * f->R,
                 c = (size_t)f->m_tilde * f->n_tilde * f->R;
    std::vector<int> key;
    key.reserve(4 + a + b + c);
    key.insert(key.end(), {f->m_tilde, f->k_tilde, f->n_tilde, f->R});
    key.insert(key.end(), f->U, f->U + a);
    key.insert(key.end(), f->V, f->V + b);
    key.insert(key.end(), f->W, f->W + c);
    {
        std::lock_guard<std::mutex> lk(g_brent_mu);
        for (const auto& k : g_brent_ok)
            if (k == key) return FMM_OK;
    }
    const int rc = fmm_check_brent(f, nullptr);
    if (rc == FMM_OK) {
        std::lock_guard<std::mutex> lk(g_brent_mu);
        if (g_brent_ok.size() < 64) g_brent_ok.push_back(std::move(key));
    }
    return rc;
}

/* flat <- levels-fold Kronecker power of fmm (levels 0: the classical
 * 1x1x1 algorithm). *owned says whether flat's arrays must be freed. */
int fmm_flatten(const fmm_t* fmm, int levels, fmm_t* flat, int* owned)
{
    static int one[1] = {1};
    *owned = 0;
    if (levels < 0 || levels > 4) return FMM_ERR_ARG;
    if (levels == 0 || fmm == nullptr) {
        *flat = fmm_t{1, 1, 1, 1, one, one, one};
        return FMM_OK;
    }
    if (!valid_fmm(fmm)) return FMM_ERR_ARG;
    if (brent_checked(fmm) != FMM_OK) return FMM_ERR_BRENT;
    if (levels == 1) {
        *flat = *fmm;
        return FMM_OK;
    }
    fmm_t cur;
    int rc = fmm_copy(fmm, &cur);
    if (rc != FMM_OK) return rc;
    for (int l = 1; l < levels; ++l) {
        fmm_t nxt;
        if ((long)cur.R * fmm->R > 1000000) { free_fmm(cur); return FMM_ERR_UNSUPPORTED; }
        rc = fmm_kron(&cur, fmm, &nxt);
        free_fmm(cur);
        if (rc != FMM_OK) return rc;
        cur = nxt;
    }
    *flat = cur;
    *owned = 1;
    return FMM_OK;
}

int fmm_alg_describe(const fmm_t* flat, std::vector<int>* table, AlgView* out)
{
    *table = build_table(flat);
    *out = view_of(*table, nullptr);
    return FMM_OK;
}

int fmm_alg_get(const fmm_t* flat, AlgView* out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FMM_ERR_CUDA;
    std::vector<int> t = build_table(flat);
    std::lock_guard<std::mutex> lk(g_mu);
    for (CachedAlg* c : g_cache)
        if (c->device == dev && c->table == t) { *out = c->view; return FMM_OK; }
    CachedAlg* c = new CachedAlg;
    c->device = dev;
    c->table = std::move(t);
    c->dtab = nullptr;
    if (cudaMalloc(&c->dtab, sizeof(int) * c->table.size()) != cudaSuccess) { delete c; return FMM_ERR_ALLOC; }
    if (cudaMemcpy(c->dtab, c->table.data(), sizeof(int) * c->table.size(), cudaMemcpyHostToDevice) !=
        cudaSuccess) {
        cudaFree(c->dtab);
        delete c;
        return FMM_ERR_CUDA;
    }
    fill_view(c);
    g_cache.push_back(c);
    *out = c->view;
    return FMM_OK;
}

static int check_gemm_args(int64_t m, int64_t n, int64_t k, const void* A, int64_t lda, const void* B,
                           int64_t ldb, const void* C, int64_t ldc)
{
    if (m < 0 || n < 0 || k < 0) return FMM_ERR_ARG;
    if (!ld_ok(lda, m) || !ld_ok(ldb, k) || !ld_ok(ldc, m)) return FMM_ERR_ARG;
    if (m > 0 && n > 0 && C == nullptr) return FMM_ERR_ARG;
    if (m > 0 && n > 0 && k > 0 && (A == nullptr || B == nullptr)) return FMM_ERR_ARG;
    return FMM_OK;
}

extern "C" int fmm_gpu_dgemm(const fmm_t* fmm, int levels, int64_t m, int64_t n, int64_t k, double alpha,
                             const double* A, int64_t lda, const double* B, int64_t ldb, double beta,
                             double* C, int64_t ldc, void* stream)
{
    int rc = check_gemm_args(m, n, k, A, lda, B, ldb, C, ldc);
    if (rc != FMM_OK) return rc;
    fmm_t flat;
    int owned = 0;
    rc = fmm_flatten(fmm, levels, &flat, &owned);
    if (rc != FMM_OK) return rc;
    AlgView alg;
    rc = fmm_alg_get(&flat, &alg);
    if (owned) free_fmm(flat);
    if (rc != FMM_OK) return rc;
    return fmm_f64_launch(alg, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, (cudaStream_t)stream);
}

extern "C" int fmm_gpu_strassen_ab_ex(double alpha, const double* A, int64_t lda, const double* B,
                                      int64_t ldb, double beta, double* C, int64_t ldc, int64_t m,
                                      int64_t n, int64_t k, fmm_t fmm)
{
    int rc = check_gemm_args(m, n, k, A, lda, B, ldb, C, ldc);
    if (rc != FMM_OK) return rc;
    /* column-major operands: the layout path of fmm_gpu_strassen_ab_gen with row stride 1 */
    return fmm_gpu_strassen_ab_gen(alpha, A, 1, std::max<int64_t>(lda, 1), B, 1, std::max<int64_t>(ldb, 1), beta, C,
                                   1, std::max<int64_t>(ldc, 1), m, n, k, fmm);
}

namespace {

/* dst[i + j*rows] = src[j + i*cols] (src: a row-major rows x cols block);
 * 32 x 32 tiles through shared memory, both sides coalesced */
__global__ void transpose_to_colmajor(const double* __restrict__ src, double* __restrict__ dst, int64_t rows,
                                      int64_t cols)
{
    __shared__ double t[32][33];
    const int64_t i0 = (int64_t)blockIdx.y * 32, j0 = (int64_t)blockIdx.x * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t i = i0 + r, j = j0 + threadIdx.x;
        if (i < rows && j < cols) t[r][threadIdx.x] = src[j + i * cols];
    }
    __syncthreads();
    for (int c = threadIdx.y; c < 32; c += blockDim.y) {
        const int64_t j = j0 + c, i = i0 + threadIdx.x;
        if (i < rows && j < cols) dst[i + j * rows] = t[threadIdx.x][c];
    }
}

/* the reverse: dst[j + i*cols] = src[i + j*rows] */
__global__ void transpose_from_colmajor(const double* __restrict__ src, double* __restrict__ dst, int64_t rows,
                                        int64_t cols)
{
    __shared__ double t[32][33];
    const int64_t i0 = (int64_t)blockIdx.y * 32, j0 = (int64_t)blockIdx.x * 32;
    for (int c = threadIdx.y; c < 32; c += blockDim.y) {
        const int64_t j = j0 + c, i = i0 + threadIdx.x;
        if (i < rows && j < cols) t[c][threadIdx.x] = src[i + j * rows];
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t i = i0 + r, j = j0 + threadIdx.x;
        if (i < rows && j < cols) dst[j + i * cols] = t[threadIdx.x][r];
    }
}

dim3 transpose_grid(int64_t rows, int64_t cols)
{
    return dim3((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32));
}

/* A host operand with element (i, j) at X[i*rs + j*cs] into the column-major
 * device array dX (rows x cols), asynchronously on st: rs == 1 is one pitched
 * copy; cs == 1 (row major, or a transposed column-major operand) is one
 * pitched copy into dtmp and a transpose on the device; any other strides
 * are gathered on the host (a pageable source: the copy has taken it when
 * cudaMemcpyAsync returns). */
int operand_to_device(const double* X, int64_t rows, int64_t cols, int64_t rs, int64_t cs, double* dX, double* dtmp,
                      cudaStream_t st)
{
    if (rows == 0 || cols == 0) return FMM_OK;
    if (rs == 1) {
        return fmm_copy2d_async(dX, sizeof(double) * rows, X, sizeof(double) * cs, sizeof(double) * rows, cols,
                                 cudaMemcpyHostToDevice, st) == cudaSuccess ? FMM_OK : FMM_ERR_CUDA;
    }
    if (cs == 1) {
        if (fmm_copy2d_async(dtmp, sizeof(double) * cols, X, sizeof(double) * rs, sizeof(double) * cols, rows,
                              cudaMemcpyHostToDevice, st) != cudaSuccess)
            return FMM_ERR_CUDA;
        transpose_to_colmajor<<<transpose_grid(rows, cols), dim3(32, 8), 0, st>>>(dtmp, dX, rows, cols);
        fmm_count_launch(1);
        return cudaGetLastError() == cudaSuccess ? FMM_OK : FMM_ERR_CUDA;
    }
    std::vector<double> h((size_t)(rows * cols));
    for (int64_t j = 0; j < cols; ++j)
        for (int64_t i = 0; i < rows; ++i) h[(size_t)(i + j * rows)] = X[i * rs + j * cs];
    return cudaMemcpyAsync(dX, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, st) == cudaSuccess
               ? FMM_OK : FMM_ERR_CUDA;
}

/* the reverse for C, on st: only the elements of the operand are written
 * (the general-strides path waits for its copy before scattering) */
int operand_to_host(const double* dX, int64_t rows, int64_t cols, double* X, int64_t rs, int64_t cs, double* dtmp,
                    cudaStream_t st)
{
    if (rows == 0 || cols == 0) return FMM_OK;
    if (rs == 1) {
        return fmm_copy2d_async(X, sizeof(double) * cs, dX, sizeof(double) * rows, sizeof(double) * rows, cols,
                                 cudaMemcpyDeviceToHost, st) == cudaSuccess ? FMM_OK : FMM_ERR_CUDA;
    }
    if (cs == 1) {
        transpose_from_colmajor<<<transpose_grid(rows, cols), dim3(32, 8), 0, st>>>(dX, dtmp, rows, cols);
        fmm_count_launch(1);
        if (cudaGetLastError() != cudaSuccess) return FMM_ERR_CUDA;
        return fmm_copy2d_async(X, sizeof(double) * rs, dtmp, sizeof(double) * cols, sizeof(double) * cols, rows,
                                 cudaMemcpyDeviceToHost, st) == cudaSuccess ? FMM_OK : FMM_ERR_CUDA;
    }
    std::vector<double> h((size_t)(rows * cols));
    if (cudaMemcpyAsync(h.data(), dX, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return FMM_ERR_CUDA;
    for (int64_t j = 0; j < cols; ++j)
        for (int64_t i = 0; i < rows; ++i) X[i * rs + j * cs] = h[(size_t)(i + j * rows)];
    return FMM_OK;
}

/* Device buffers of the host-buffer calls of any layout (fmm_gpu_strassen_ab_ex,
 * fmm_gpu_strassen_ab_gen and the split form's non-column-major path), per
 * device: grow-only, kept between calls so a call allocates nothing once
 * warm, freed by fmm_gpu_release_host_buffers; and one non-blocking stream per
 * device that the calls' copies and kernels run on. */
struct GenBuffers {
    void* p[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};   /* A, B, C, transpose scratch, split workspace */
    size_t have[5] = {0, 0, 0, 0, 0};
    cudaStream_t st = nullptr;
};
std::mutex g_gen_mu;
GenBuffers g_gen[64];

/* buffer x of at least `need` bytes (the stream is idle between calls) */
int gen_buffer(GenBuffers& b, int x, size_t need, void** out)
{
    need = std::max<size_t>(need, 256);
    if (b.have[x] < need) {
        if (b.p[x]) cudaFree(b.p[x]);
        b.p[x] = nullptr;
        b.have[x] = 0;
        if (cudaMalloc(&b.p[x], need) != cudaSuccess) return FMM_ERR_ALLOC;
        b.have[x] = need;
    }
    *out = b.p[x];
    return FMM_OK;
}

int gen_device(GenBuffers** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return FMM_ERR_CUDA;
    GenBuffers& b = g_gen[dev];
    if (b.st == nullptr && cudaStreamCreateWithFlags(&b.st, cudaStreamNonBlocking) != cudaSuccess) return FMM_ERR_CUDA;
    *out = &b;
    return FMM_OK;
}

/* needs a transpose scratch: some operand is row-major (or transposed) */
bool gen_needs_tmp(int64_t rsa, int64_t csa, int64_t rsb, int64_t csb, int64_t rsc, int64_t csc)
{
    return (rsa != 1 && csa == 1) || (rsb != 1 && csb == 1) || (rsc != 1 && csc == 1);
}

}  // namespace

extern "C" int fmm_gpu_strassen_ab_gen(double alpha, const double* A, int64_t rsa, int64_t csa, const double* B,
                                       int64_t rsb, int64_t csb, double beta, double* C, int64_t rsc,
                                       int64_t csc, int64_t m, int64_t n, int64_t k, fmm_t fmm)
{
    if (m < 0 || n < 0 || k < 0) return FMM_ERR_ARG;
    if (rsa < 1 || csa < 1 || rsb < 1 || csb < 1 || rsc < 1 || csc < 1) return FMM_ERR_ARG;
    if (m > 0 && n > 0 && C == nullptr) return FMM_ERR_ARG;
    if (m > 0 && n > 0 && k > 0 && (A == nullptr || B == nullptr)) return FMM_ERR_ARG;
    if (m == 0 || n == 0) return FMM_OK;
    std::lock_guard<std::mutex> lk(g_gen_mu);
    GenBuffers* b = nullptr;
    int rc = gen_device(&b);
    if (rc != FMM_OK) return rc;
    const int64_t ka = k > 0 ? k : 1;
    const size_t tmp = sizeof(double) * (size_t)std::max(std::max(m * ka, ka * n), m * n);
    void *dA = nullptr, *dB = nullptr, *dC = nullptr, *dT = nullptr;
    if ((rc = gen_buffer(*b, 0, sizeof(double) * (size_t)(m * ka), &dA)) != FMM_OK ||
        (rc = gen_buffer(*b, 1, sizeof(double) * (size_t)(ka * n), &dB)) != FMM_OK ||
        (rc = gen_buffer(*b, 2, sizeof(double) * (size_t)(m * n), &dC)) != FMM_OK ||
        (gen_needs_tmp(rsa, csa, rsb, csb, rsc, csc) && (rc = gen_buffer(*b, 3, tmp, &dT)) != FMM_OK))
        return rc;
    if (k > 0) rc = operand_to_device(A, m, k, rsa, csa, (double*)dA, (double*)dT, b->st);
    if (rc == FMM_OK && k > 0) rc = operand_to_device(B, k, n, rsb, csb, (double*)dB, (double*)dT, b->st);
    if (rc == FMM_OK) rc = operand_to_device(C, m, n, rsc, csc, (double*)dC, (double*)dT, b->st);
    if (rc == FMM_OK)
        rc = fmm_gpu_dgemm(&fmm, 1, m, n, k, alpha, (double*)dA, m, (double*)dB, ka, beta, (double*)dC, m, b->st);
    if (rc == FMM_OK) rc = operand_to_host((double*)dC, m, n, C, rsc, csc, (double*)dT, b->st);
    if (cudaStreamSynchronize(b->st) != cudaSuccess && rc == FMM_OK) rc = FMM_ERR_CUDA;
    if (rc == FMM_OK) rc = fmm_device_error_status();
    return rc;
}

extern "C" int fmm_gpu_strassen_ab(double alpha, const double* A, int64_t lda, const double* B, int64_t ldb,
                                   double beta, double* C, int64_t ldc, int64_t m, int64_t n, int64_t k)
{
    return fmm_gpu_strassen_ab_ex(alpha, A, lda, B, ldb, beta, C, ldc, m, n, k, STRASSEN_FMM);
}

extern "C" size_t fmm_gpu_split_workspace_size(const fmm_t* fmm, int levels, int64_t m, int64_t n, int64_t k,
                                               int slices)
{
    return fmm_gpu_split_workspace_size_fmt(fmm, levels, m, n, k, slices, FMM_SPLIT_BF16);
}

extern "C" size_t fmm_gpu_split_workspace_size_fmt(const fmm_t* fmm, int levels, int64_t m, int64_t n, int64_t k,
                                                   int slices, int format)
{
    if (format != FMM_SPLIT_BF16 && format != FMM_SPLIT_FP8_E4M3) return 0;
    if (m < 0 || n < 0 || k < 0 || slices < 2 || slices > (format ? 12 : 8)) return 0;
    fmm_t flat;
    int owned = 0;
    if (fmm_flatten(fmm, levels, &flat, &owned) != FMM_OK) return 0;
    AlgView v;
    v.mt = flat.m_tilde; v.kt = flat.k_tilde; v.nt = flat.n_tilde; v.R = flat.R;
    size_t b = fmm_split_ws_bytes(v, m, n, k, slices, format);
    if (owned) free_fmm(flat);
    return b;
}

extern "C" int fmm_gpu_split_dgemm(const fmm_t* fmm, int levels, int64_t m, int64_t n, int64_t k,
                                   double alpha, const double* A, int64_t lda, const double* B, int64_t ldb,
                                   double beta, double* C, int64_t ldc, int slices, void* workspace,
                                   size_t workspace_bytes, void* stream)
{
    return fmm_gpu_split_dgemm_fmt(fmm, levels, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, slices,
                                   FMM_SPLIT_BF16, workspace, workspace_bytes, stream);
}

extern "C" int fmm_gpu_split_strassen_ab_ex(double alpha, const double* A, int64_t lda, const double* B,
                                            int64_t ldb, double beta, double* C, int64_t ldc, int64_t m,
                                            int64_t n, int64_t k, fmm_t fmm, int levels, int slices, int format)
{
    int rc = check_gemm_args(m, n, k, A, lda, B, ldb, C, ldc);
    if (rc != FMM_OK) return rc;
    if (format != FMM_SPLIT_BF16 && format != FMM_SPLIT_FP8_E4M3) return FMM_ERR_ARG;
    if (slices < 2 || slices > (format ? 12 : 8)) return FMM_ERR_ARG;
    fmm_t flat;
    int owned = 0;
    rc = fmm_flatten(levels > 0 ? &fmm : nullptr, levels, &flat, &owned);
    if (rc != FMM_OK) return rc;
    AlgView alg;
    rc = fmm_alg_get(&flat, &alg);
    if (owned) free_fmm(flat);
    if (rc != FMM_OK) return rc;
    if (fmm_device_error_word() == nullptr) return FMM_ERR_CUDA;
    return fmm_split_host(alg, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, slices, format);
}

extern "C" void fmm_gpu_release_host_buffers(void)
{
    fmm_split_host_release();
    std::lock_guard<std::mutex> lk(g_gen_mu);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
    GenBuffers& b = g_gen[dev];
    if (b.st) cudaStreamSynchronize(b.st);
    for (int x = 0; x < 5; ++x) {
        if (b.p[x]) cudaFree(b.p[x]);
        b.p[x] = nullptr;
        b.have[x] = 0;
    }
}

void fmm_touch_host(const void* p, size_t bytes)
{
    static const size_t page = []() {
        const long v = sysconf(_SC_PAGESIZE);
        return v > 0 ? (size_t)v : (size_t)4096;
    }();
    if (p == nullptr || bytes == 0) return;
    const volatile uint8_t* b = (const volatile uint8_t*)p;
    /* from the page holding the first byte to the page holding the last */
    const size_t lead = (uintptr_t)p % page;
    uint8_t sink = 0;
    for (size_t off = 0; off < bytes + lead; off += page) sink ^= b[off > lead ? off - lead : 0];
    sink ^= b[bytes - 1];
    (void)sink;
}

/* ---------------------------------------------------------------------------
 * Pinned host buffers on transparent huge pages.
 *
 * The host-buffer entry points copy the caller's operands over the host link.
 * A copy engine reading pinned memory translates every page it touches; with
 * small pages a 2 GiB operand spans tens of thousands of translations, and a
 * copy that starts after the host has been idle for a few seconds ran at a
 * quarter of the link's rate on a GB300 host (64 KiB pages: 40.5 ms against
 * 10.2 ms for 2 GiB; cudaHostAlloc memory 13.7 ms), while the same buffer on
 * huge pages stayed at 10.2 ms. fmm_gpu_host_alloc maps anonymous memory
 * aligned to the huge-page size, asks for huge pages (madvise MADV_HUGEPAGE,
 * honoured where the kernel's transparent huge pages are "always" or
 * "madvise"), touches it so the pages exist, and page-locks it for the GPU
 * (cudaHostRegister).
 * ------------------------------------------------------------------------- */
namespace {
struct HostMap {
    void* base;
    size_t len;
};
std::mutex g_hostmap_mu;
std::map<void*, HostMap> g_hostmap;

size_t huge_page_bytes()
{
    static size_t hp = 0;
    static std::once_flag once;
    std::call_once(once, []() {
        hp = 2u << 20;
        if (FILE* f = fopen("/sys/kernel/mm/transparent_hugepage/hpage_pmd_size", "r")) {
            unsigned long long v = 0;
            if (fscanf(f, "%llu", &v) == 1 && v >= 4096 && (v & (v - 1)) == 0) hp = (size_t)v;
            fclose(f);
        }
    });
    return hp;
}
}  // namespace

extern "C" int fmm_gpu_host_alloc(size_t bytes, void** ptr)
{
    if (ptr == nullptr) return FMM_ERR_ARG;
    *ptr = nullptr;
    if (bytes == 0) return FMM_ERR_ARG;
    const size_t page = (size_t)sysconf(_SC_PAGESIZE);
    const size_t hp = huge_page_bytes();
    /* huge pages only where the buffer holds at least one; otherwise plain pages */
    const size_t align = bytes >= hp ? hp : page;
    const size_t len = (bytes + align - 1) / align * align;
    const size_t map_len = len + align;
    void* base = mmap(nullptr, map_len, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
    if (base == MAP_FAILED) return FMM_ERR_ALLOC;
    uint8_t* p = (uint8_t*)(((uintptr_t)base + align - 1) / align * align);
#ifdef MADV_HUGEPAGE
    if (align == hp) madvise(p, len, MADV_HUGEPAGE);
#endif
    memset(p, 0, len);
    /* where the first touch fell back to small pages (no free huge page at
     * fault time), ask the kernel to collapse the range now (Linux 6.1+;
     * MADV_COLLAPSE, 25, compacts memory to find huge pages; an older kernel
     * refuses it and the small pages stay) */
    if (align == hp) madvise(p, len, 25);
    if (cudaHostRegister(p, len, cudaHostRegisterDefault) != cudaSuccess) {
        cudaGetLastError();
        munmap(base, map_len);
        return FMM_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lk(g_hostmap_mu);
    g_hostmap[p] = HostMap{base, map_len};
    *ptr = p;
    return FMM_OK;
}

extern "C" int fmm_gpu_host_free(void* ptr)
{
    if (ptr == nullptr) return FMM_OK;
    HostMap h;
    {
        std::lock_guard<std::mutex> lk(g_hostmap_mu);
        auto it = g_hostmap.find(ptr);
        if (it == g_hostmap.end()) return FMM_ERR_ARG;
        h = it->second;
        g_hostmap.erase(it);
    }
    const cudaError_t e = cudaHostUnregister(ptr);
    munmap(h.base, h.len);
    return e == cudaSuccess ? FMM_OK : FMM_ERR_CUDA;
}

extern "C" int fmm_gpu_split_strassen_ab_gen(double alpha, const double* A, int64_t rsa, int64_t csa,
                                             const double* B, int64_t rsb, int64_t csb, double beta, double* C,
                                             int64_t rsc, int64_t csc, int64_t m, int64_t n, int64_t k, fmm_t fmm,
                                             int levels, int slices, int format)
{
    if (m < 0 || n < 0 || k < 0) return FMM_ERR_ARG;
    if (rsa < 1 || csa < 1 || rsb < 1 || csb < 1 || rsc < 1 || csc < 1) return FMM_ERR_ARG;
    if (m > 0 && n > 0 && C == nullptr) return FMM_ERR_ARG;
    if (m > 0 && n > 0 && k > 0 && (A == nullptr || B == nullptr)) return FMM_ERR_ARG;
    if (format != FMM_SPLIT_BF16 && format != FMM_SPLIT_FP8_E4M3) return FMM_ERR_ARG;
    if (slices < 2 || slices > (format ? 12 : 8)) return FMM_ERR_ARG;
    if (m == 0 || n == 0) return FMM_OK;
    /* column-major operands: the overlapped host-buffer pipeline */
    if (rsa == 1 && rsb == 1 && rsc == 1 && csa >= m && csb >= std::max<int64_t>(k, 1) && csc >= m)
        return fmm_gpu_split_strassen_ab_ex(alpha, A, csa, B, csb, beta, C, csc, m, n, k, fmm, levels, slices,
                                            format);
    /* other layouts: column-major device copies (transposed on the device or
     * gathered on the host), the device call, C written back in place */
    const fmm_t* pf = levels > 0 ? &fmm : nullptr;
    const size_t wsb = fmm_gpu_split_workspace_size_fmt(pf, levels, m, n, k, slices, format);
    if (wsb == 0) return FMM_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_gen_mu);
    GenBuffers* b = nullptr;
    int rc = gen_device(&b);
    if (rc != FMM_OK) return rc;
    const int64_t ka = k > 0 ? k : 1;
    const size_t tmp = sizeof(double) * (size_t)std::max(std::max(m * ka, ka * n), m * n);
    void *dA = nullptr, *dB = nullptr, *dC = nullptr, *dT = nullptr, *ws = nullptr;
    if ((rc = gen_buffer(*b, 0, sizeof(double) * (size_t)(m * ka), &dA)) != FMM_OK ||
        (rc = gen_buffer(*b, 1, sizeof(double) * (size_t)(ka * n), &dB)) != FMM_OK ||
        (rc = gen_buffer(*b, 2, sizeof(double) * (size_t)(m * n), &dC)) != FMM_OK ||
        (gen_needs_tmp(rsa, csa, rsb, csb, rsc, csc) && (rc = gen_buffer(*b, 3, tmp, &dT)) != FMM_OK) ||
        (rc = gen_buffer(*b, 4, wsb, &ws)) != FMM_OK)
        return rc;
    if (k > 0) rc = operand_to_device(A, m, k, rsa, csa, (double*)dA, (double*)dT, b->st);
    if (rc == FMM_OK && k > 0) rc = operand_to_device(B, k, n, rsb, csb, (double*)dB, (double*)dT, b->st);
    if (rc == FMM_OK) rc = operand_to_device(C, m, n, rsc, csc, (double*)dC, (double*)dT, b->st);
    if (rc == FMM_OK)
        rc = fmm_gpu_split_dgemm_fmt(pf, levels, m, n, k, alpha, (double*)dA, m, (double*)dB, ka, beta, (double*)dC,
                                     m, slices, format, ws, b->have[4], b->st);
    if (rc == FMM_OK) rc = operand_to_host((double*)dC, m, n, C, rsc, csc, (double*)dT, b->st);
    if (cudaStreamSynchronize(b->st) != cudaSuccess && rc == FMM_OK) rc = FMM_ERR_CUDA;
    if (rc == FMM_OK) rc = fmm_device_error_status();
    return rc;
}

extern "C" int fmm_gpu_split_dgemm_fmt(const fmm_t* fmm, int levels, int64_t m, int64_t n, int64_t k,
                                       double alpha, const double* A, int64_t lda, const double* B, int64_t ldb,
                                       double beta, double* C, int64_t ldc, int slices, int format,
                                       void* workspace, size_t workspace_bytes, void* stream)
{
    int rc = check_gemm_args(m, n, k, A, lda, B, ldb, C, ldc);
    if (rc != FMM_OK) return rc;
    if (format != FMM_SPLIT_BF16 && format != FMM_SPLIT_FP8_E4M3) return FMM_ERR_ARG;
    if (slices < 2 || slices > (format ? 12 : 8)) return FMM_ERR_ARG;
    fmm_t flat;
    int owned = 0;
    rc = fmm_flatten(fmm, levels, &flat, &owned);
    if (rc != FMM_OK) return rc;
    AlgView alg;
    rc = fmm_alg_get(&flat, &alg);
    if (owned) free_fmm(flat);
    if (rc != FMM_OK) return rc;
    if (fmm_device_error_word() == nullptr) return FMM_ERR_CUDA;
    return fmm_split_launch(alg, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, slices, format, workspace,
                            workspace_bytes, (cudaStream_t)stream);
}
