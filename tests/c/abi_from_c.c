/* The GB300 library used from C the way a BLIS-side shim would: only the
 * public header, linked against libfmm_gb300.so. Host-only entry points are
 * exercised (coefficient files, Brent check, Kronecker product, status
 * strings, argument errors); no GPU is needed. Prints "ok" on success. */
#include <stdio.h>
#include <string.h>

#include "fmm_gb300.h"

static int fails = 0;
#define CHECK(c)                                                   \
    do {                                                           \
        if (!(c)) { fprintf(stderr, "failed: %s\n", #c); ++fails; } \
    } while (0)

int main(int argc, char** argv)
{
    if (argc < 2) { fprintf(stderr, "usage: abi_from_c <coeff dir>\n"); return 2; }
    char path[4096];
    snprintf(path, sizeof path, "%s/222.txt", argv[1]);

    /* the reference's by-value reader and STRASSEN_FMM */
    fmm_t f = new_fmm(path);
    CHECK(f.R == 7 && f.m_tilde == 2 && f.k_tilde == 2 && f.n_tilde == 2);
    CHECK(STRASSEN_FMM.R == 7);
    for (int i = 0; i < 4 * 7; ++i) CHECK(f.U[i] == STRASSEN_FMM.U[i]);
    long bad = -1;
    CHECK(fmm_check_brent(&f, &bad) == FMM_OK && bad == 0);

    /* two levels by the Kronecker product: 49 products, still exact */
    fmm_t f2;
    CHECK(fmm_kron(&f, &f, &f2) == FMM_OK);
    CHECK(f2.R == 49 && f2.m_tilde == 4);
    CHECK(fmm_check_brent(&f2, &bad) == FMM_OK && bad == 0);
    free_fmm(f2);

    /* a missing file is a status, not a crash */
    fmm_t g;
    CHECK(fmm_load("/nonexistent/fmm.txt", &g) != FMM_OK);
    CHECK(strlen(fmm_status_string(FMM_ERR_ARG)) > 0);

    /* argument checks come before any device work */
    double a[16] = {0};
    CHECK(fmm_gpu_strassen_ab_ex(1.0, a, 3, a, 4, 1.0, a, 4, 4, 4, 4, f) == FMM_ERR_ARG);   /* lda < m */
    CHECK(fmm_gpu_split_strassen_ab_ex(1.0, a, 4, a, 4, 1.0, a, 4, 4, 4, 4, f, 1, 9, FMM_SPLIT_BF16) == FMM_ERR_ARG);
    CHECK(fmm_gpu_split_strassen_ab_gen(1.0, a, 1, 4, a, 1, 4, 1.0, a, 1, 4, 4, 4, 4, f, 1, 6, 7) == FMM_ERR_ARG);
    CHECK(fmm_gpu_split_workspace_size(&f, 1, 64, 64, 64, 6) > 0);
    CHECK(fmm_gpu_split_workspace_size_fmt(&f, 1, 64, 64, 64, 13, FMM_SPLIT_FP8_E4M3) == 0);
    CHECK(fmm_gpu_set_split_pair_rows(fmm_gpu_set_split_pair_rows(1024)) == 1024);

    free_fmm(f);
    if (fails) return 1;
    printf("ok\n");
    return 0;
}
