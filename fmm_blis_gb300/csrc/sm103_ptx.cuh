/*
 * Thin inline-PTX wrappers for the sm_103a features the split-precision GEMM
 * uses: mbarriers with time-bounded waits, TMA tiled loads, and the tcgen05
 * tensor-memory (TMEM) / MMA instructions.
 *
 * Every wait is bounded by the global timer: after kWaitLimitNs the waiting
 * thread records an error code in the device error word and returns false,
 * so a kernel whose partner never arrives ends instead of hanging the GPU.
 */
#ifndef SM103_PTX_CUH
#define SM103_PTX_CUH

#include <stdint.h>

namespace sm103 {

constexpr uint64_t kWaitLimitNs = 2000000000ull; /* 2 s */

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}"
                 ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}"
                 ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return ok != 0;
}

/* Waits for the phase with the given parity to complete. Returns false (and
 * sets *err to code if it was 0) when the wait exceeded the time limit or
 * another thread already flagged an abort. */
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                          int* err, int code)
{
    if (mbar_try_wait(bar, parity)) return true;
    uint64_t t0 = globaltimer();
    for (uint32_t it = 0;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 255u) == 255u) {
            if (*abort_flag) return false;
            if (globaltimer() - t0 > kWaitLimitNs) {
                *abort_flag = 1;
                atomicCAS(err, 0, code);
                return false;
            }
        }
    }
}

/* ---- clusters (CTA pairs) ---- */

__device__ __forceinline__ uint32_t cluster_ctarank()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

/* all threads of both CTAs of the cluster */
__device__ __forceinline__ void cluster_sync()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

/* the shared::cluster address of the same shared-memory location in CTA `rank` */
__device__ __forceinline__ uint32_t mapa(uint32_t smem_addr, uint32_t rank)
{
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_addr), "r"(rank));
    return r;
}

/* arrive on an mbarrier of a CTA of the cluster, ordering this thread's
 * earlier loads and stores (also to other CTAs' shared memory) before it */
__device__ __forceinline__ void mbar_arrive_release_cluster(uint32_t cluster_addr)
{
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cluster_addr) : "memory");
}

/* the same wait on a barrier given by its shared-memory address */
__device__ __forceinline__ bool mbar_wait_acq_cluster_u32(uint32_t bar, uint32_t parity, volatile int* abort_flag,
                                                          int* err, int code);

__device__ __forceinline__ uint32_t ld_shared_u32(uint32_t addr)
{
    uint32_t v;
    asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(addr) : "memory");
    return v;
}

/* store to the shared memory of a CTA of the cluster (address from mapa) */
__device__ __forceinline__ void st_shared_cluster_u32(uint32_t cluster_addr, uint32_t v)
{
    asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(cluster_addr), "r"(v) : "memory");
}

/* mbar_wait for a phase completed by arrivals (with release.cluster) from
 * either CTA of the cluster: acquire at cluster scope */
__device__ __forceinline__ bool mbar_try_wait_acq_cluster(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_try_wait_acq_cluster_u32(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_acq_cluster(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                                      int* err, int code)
{
    if (mbar_try_wait_acq_cluster(bar, parity)) return true;
    uint64_t t0 = globaltimer();
    for (uint32_t it = 0;; ++it) {
        if (mbar_try_wait_acq_cluster(bar, parity)) return true;
        if ((it & 255u) == 255u) {
            if (*abort_flag) return false;
            if (globaltimer() - t0 > kWaitLimitNs) {
                *abort_flag = 1;
                atomicCAS(err, 0, code);
                return false;
            }
        }
    }
}

__device__ __forceinline__ bool mbar_wait_acq_cluster_u32(uint32_t bar, uint32_t parity, volatile int* abort_flag,
                                                          int* err, int code)
{
    if (mbar_try_wait_acq_cluster_u32(bar, parity)) return true;
    uint64_t t0 = globaltimer();
    for (uint32_t it = 0;; ++it) {
        if (mbar_try_wait_acq_cluster_u32(bar, parity)) return true;
        if ((it & 255u) == 255u) {
            if (*abort_flag) return false;
            if (globaltimer() - t0 > kWaitLimitNs) {
                *abort_flag = 1;
                atomicCAS(err, 0, code);
                return false;
            }
        }
    }
}

/* 2-D TMA tiled load into this CTA's shared memory whose completion is
 * counted on an mbarrier of either CTA of the pair (bar_cluster from mapa) */
__device__ __forceinline__ void tma_load_2d_pair(void* dst, const void* tmap, uint32_t bar_cluster, int x, int y)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.cta_group::2"
        " [%0], [%1, {%3, %4}], [%2];"
        ::"r"(smem_u32(dst)), "l"(tmap), "r"(bar_cluster), "r"(x), "r"(y)
        : "memory");
}

/* arrive on an mbarrier of a CTA of the cluster (address from mapa) */
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t cluster_addr)
{
    /* default .release.cta: what the arrive publishes is ordered by the
     * tcgen05 fences (TMEM reads done), not by generic memory, so the
     * cluster-scope release (a fence behind every outstanding Z reduction)
     * is not needed */
    asm volatile("mbarrier.arrive.shared::cluster.b64 _, [%0];" ::"r"(cluster_addr) : "memory");
}

/* 2-D TMA tiled load into shared memory, completion on an mbarrier. */
__device__ __forceinline__ void tma_load_2d(void* dst, const void* tmap, uint64_t* bar, int x, int y)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%3, %4}], [%2];"
        ::"r"(smem_u32(dst)), "l"(tmap), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

__device__ __forceinline__ void prefetch_tmap(const void* tmap)
{
    asm volatile("prefetch.tensormap [%0];" ::"l"(tmap) : "memory");
}

/* ---- tcgen05 ---- */

__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(smem_u32(dst_smem)), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tmem_relinquish()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

/* D[tmem] (+)= A[smem desc] * B[smem desc], kind::f16 (BF16 in, FP32 accumulate). */
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                         uint32_t idesc, uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.u32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                 ::"r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
                 : "memory");
}

/* CTA-pair forms: the allocation is made by one warp in each CTA of the
 * pair (same columns in both); the MMA, issued by the even CTA, multiplies
 * M = 256 rows (128 in each CTA's shared memory) by N columns (half in
 * each) into both CTAs' TMEM; the commit arrives on the barrier at the same
 * offset in both CTAs. */
__device__ __forceinline__ void tmem_alloc_pair(uint32_t* dst_smem, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(smem_u32(dst_smem)), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tmem_relinquish_pair()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc_pair(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mma_bf16_pair(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                              uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.u32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                 ::"r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
                 : "memory");
}

__device__ __forceinline__ void mma_f8_pair(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                            uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.u32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}"
                 ::"r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
                 : "memory");
}

/* arrive on `bar` in both CTAs of the pair once all previously issued
 * tcgen05.mma of this thread have completed */
__device__ __forceinline__ void mma_commit_pair(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;"
                 ::"r"(smem_u32(bar)), "h"((unsigned short)3) : "memory");
}

/* D[tmem] (+)= A[smem desc] * B[smem desc], kind::f8f6f4 (FP8 in, FP32 accumulate). */
__device__ __forceinline__ void mma_f8(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                       uint32_t idesc, uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.u32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}"
                 ::"r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
                 : "memory");
}

/* Arrive on an mbarrier once all previously issued tcgen05.mma of this
 * thread have completed. */
__device__ __forceinline__ void mma_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 ::"r"(smem_u32(bar)) : "memory");
}

/* Shared-memory matrix descriptor, K-major operand with 128-byte swizzle:
 * 8-row groups 1024 bytes apart, start address encoded >> 4. */
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);        /* start address */
    d |= (uint64_t)1 << 16;                          /* leading byte offset (unused for SW128 K-major) */
    d |= (uint64_t)(1024u >> 4) << 32;               /* stride byte offset */
    d |= (uint64_t)1 << 46;                          /* descriptor version (sm_100 family) */
    d |= (uint64_t)2 << 61;                          /* 128-byte swizzle */
    return d;
}

/* Instruction descriptor for kind::f16: BF16 A and B (both K-major), FP32 D. */
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N)
{
    return (1u << 4)                       /* D format: F32 */
         | (1u << 7)                       /* A format: BF16 */
         | (1u << 10)                      /* B format: BF16 */
         | ((uint32_t)(N >> 3) << 17)      /* N / 8 */
         | ((uint32_t)(M >> 4) << 24);     /* M / 16 */
}

/* Instruction descriptor for kind::f8f6f4: E4M3 A and B (format 0, both
 * K-major), FP32 D. */
__host__ __device__ constexpr uint32_t idesc_e4m3_f32(int M, int N)
{
    return (1u << 4)                       /* D format: F32 */
         | ((uint32_t)(N >> 3) << 17)      /* N / 8 */
         | ((uint32_t)(M >> 4) << 24);     /* M / 16 */
}

#define SM103_TMEM_LD_X8(taddr, r)                                                               \
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"          \
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),       \
                   "=r"(r[6]), "=r"(r[7])                                                        \
                 : "r"(taddr))

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

}  // namespace sm103

#endif
