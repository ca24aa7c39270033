/*
 * BLIS-side drop-in: the reference's object-API entry points, implemented on
 * the GB300 library. A BLIS application (such as the reference's own test
 * driver, test/test_strassen_oapi.c) compiles unchanged against the
 * reference's bli_fmm.h and links this file, libfmm_gb300.so and libblis
 * instead of the reference's libfmm.a and fmm_blis plugin:
 *
 *     cc -c bli_strassen_ab_gpu.c -I<blis include dir> -I<repo>/include
 *     cc app.o bli_strassen_ab_gpu.o -L<repo>/fmm_blis_gb300 -lfmm_gb300 libblis.a -fopenmp -lm
 *
 * Replaces frame/base/bli_strassen_ab.c:123-300 (bli_strassen_ab_ex and
 * bli_strassen_ab, declared at frame/include/bli_fmm.h:74-89). new_fmm,
 * free_fmm, STRASSEN_FMM and bl_clock come from libfmm_gb300.so with the
 * reference's signatures (frame/include/bli_fmm.h:69-70, 205). Operands are
 * read through BLIS's obj_t accessors, as the reference reads them
 * (bli_strassen_ab.c:165-172); the GPU library stages host buffers itself.
 * Errors follow the reference: a message, then bli_abort()
 * (bli_strassen_ab.c:130-135).
 *
 * Plugin registration (plugin/bli_plugin_register.c:43-64): as in the
 * reference, the first bli_strassen_ab_ex call registers a kernel ID with
 * BLIS's global kernel structure (bli_gks_register_ukr) and installs the
 * kernel in the contexts; later calls look it up in the active context
 * (bli_strassen_ab.c:125-137, 219) and call it. Here the registered kernel
 * (FMM_BLIS_GEMM_UKR, double precision slot) is the whole GPU FMM, since
 * packing and the multi-C epilogue run inside it; the registration is done
 * once under pthread_once (the reference's static flag is unsynchronised).
 *
 * Compiles only where BLIS's installed headers are (it is not part of
 * libfmm_gb300.so, which has no BLIS dependency).
 */
#include "blis.h"
#include "fmm_gb300.h"

#include <pthread.h>
#include <stdio.h>

/* element (i, j) of op(X) sits at buf[i*rs + j*cs]: a transposed object
 * swaps its strides */
static void op_strides(const obj_t* X, int64_t* rs, int64_t* cs)
{
    *rs = (int64_t)bli_obj_row_stride(X);
    *cs = (int64_t)bli_obj_col_stride(X);
    if (bli_obj_has_trans(X)) {
        int64_t t = *rs;
        *rs = *cs;
        *cs = t;
    }
}

static double real_of(const obj_t* s)
{
    double re = 0.0, im = 0.0;
    bli_getsc(s, &re, &im);
    return re;
}

/* the GPU FMM on BLIS objects: the kernel the plugin registers */
static void gpu_fmm_obj(obj_t* alpha, obj_t* A, obj_t* B, obj_t* beta, obj_t* C, fmm_t fmm)
{
    if (bli_obj_dt(A) != BLIS_DOUBLE || bli_obj_dt(B) != BLIS_DOUBLE || bli_obj_dt(C) != BLIS_DOUBLE) {
        fprintf(stderr, "bli_strassen_ab_ex: the GB300 library computes in double precision only\n");
        bli_abort();
    }
    const int64_t m = (int64_t)bli_obj_length(C), n = (int64_t)bli_obj_width(C);
    const int64_t k = (int64_t)bli_obj_width_after_trans(A);
    if ((int64_t)bli_obj_length_after_trans(A) != m || (int64_t)bli_obj_length_after_trans(B) != k ||
        (int64_t)bli_obj_width_after_trans(B) != n) {
        fprintf(stderr, "bli_strassen_ab_ex: operand dimensions do not conform\n");
        bli_abort();
    }
    int64_t rsa, csa, rsb, csb, rsc, csc;
    op_strides(A, &rsa, &csa);
    op_strides(B, &rsb, &csb);
    op_strides(C, &rsc, &csc);
    const int st = fmm_gpu_strassen_ab_gen(real_of(alpha), (const double*)bli_obj_buffer_at_off(A), rsa, csa,
                                           (const double*)bli_obj_buffer_at_off(B), rsb, csb, real_of(beta),
                                           (double*)bli_obj_buffer_at_off(C), rsc, csc, m, n, k, fmm);
    if (st != FMM_OK) {
        fprintf(stderr, "bli_strassen_ab_ex: fmm_gpu_strassen_ab_gen: %s\n", fmm_status_string(st));
        bli_abort();
    }
}

typedef void (*fmm_obj_ft)(obj_t*, obj_t*, obj_t*, obj_t*, obj_t*, fmm_t);

/* BLIS kernel ID of the GPU FMM (the reference's plugin keeps its kernel
 * IDs in globals of these names, plugin/bli_plugin_register.c:40-41) */
siz_t FMM_BLIS_GEMM_UKR;

/* plugin/bli_plugin_register.c:43-64: registers the kernel ID and installs
 * the GPU FMM (double precision) in every context BLIS has set up */
err_t bli_plugin_register_fmm_blis(void)
{
    err_t err = bli_gks_register_ukr(&FMM_BLIS_GEMM_UKR);
    if (err != BLIS_SUCCESS) return err;
    func_t f;
    bli_func_init(&f, NULL, (void_fp)gpu_fmm_obj, NULL, NULL);
    for (int id = 0; id < (int)BLIS_NUM_ARCHS; ++id) {
        cntx_t* cntx = (cntx_t*)bli_gks_lookup_id((arch_t)id);
        if (cntx != NULL) bli_cntx_set_ukr((ukr_t)FMM_BLIS_GEMM_UKR, &f, cntx);
    }
    return BLIS_SUCCESS;
}

static pthread_once_t g_register_once = PTHREAD_ONCE_INIT;
static err_t g_register_err = BLIS_FAILURE;

static void register_once(void)
{
    g_register_err = bli_plugin_register_fmm_blis();
}

void bli_strassen_ab_ex(obj_t* alpha, obj_t* A, obj_t* B, obj_t* beta, obj_t* C, fmm_t fmm)
{
    bli_init_once();
    pthread_once(&g_register_once, register_once);
    if (g_register_err != BLIS_SUCCESS) {
        printf("error %d\n", (int)g_register_err);
        bli_abort();
    }
    const func_t* f = bli_cntx_get_ukrs((ukr_t)FMM_BLIS_GEMM_UKR, bli_gks_query_cntx());
    fmm_obj_ft kernel = (fmm_obj_ft)bli_func_get_dt(BLIS_DOUBLE, f);
    if (kernel == NULL) {
        fprintf(stderr, "bli_strassen_ab_ex: no GPU FMM kernel registered in the active context\n");
        bli_abort();
    }
    kernel(alpha, A, B, beta, C, fmm);
}

void bli_strassen_ab(obj_t* alpha, obj_t* A, obj_t* B, obj_t* beta, obj_t* C)
{
    bli_strassen_ab_ex(alpha, A, B, beta, C, STRASSEN_FMM);
}
