/* ORACLE -- test infrastructure only. Runs the reference's own FMM,
 * bli_strassen_ab_ex (frame/base/bli_strassen_ab.c:123), on operands read
 * from a file and writes the resulting C, so that the reference's outputs can
 * be kept as golden fixtures. Built by oracle/build_ref.sh against the
 * reference build in oracle/_ref/; never part of the product.
 *
 * Input file (little-endian): int64 m, n, k, m~, k~, n~, R; then int32 U
 * (m~k~ rows x R), V (k~n~ x R), W (m~n~ x R), row-major as in the coefficient
 * files; then float64 A (m x k), B (k x n), C (m x n), column-major with
 * leading dimensions m, k, m. Output file: float64 C after
 * C := C + A*B (alpha = beta = 1, the semantics the reference honours).
 *
 * The fmm_t is filled field by field (m_tilde, n_tilde, k_tilde as the driver
 * uses them), not through the reference's reader, so the reader's header-order
 * and line-length defects do not enter. */
#include "blis.h"
#include "bli_fmm.h"

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

static int read_all(FILE* f, void* p, size_t bytes)
{
    return bytes == 0 || fread(p, 1, bytes, f) == bytes;
}

int main(int argc, char** argv)
{
    if (argc != 3) {
        fprintf(stderr, "usage: %s <input> <output>\n", argv[0]);
        return 2;
    }
    FILE* in = fopen(argv[1], "rb");
    if (!in) { perror(argv[1]); return 2; }
    int64_t h[7];
    if (!read_all(in, h, sizeof h)) { fprintf(stderr, "short header\n"); return 2; }
    const int64_t m = h[0], n = h[1], k = h[2];
    fmm_t fmm;
    fmm.m_tilde = (int)h[3];
    fmm.k_tilde = (int)h[4];
    fmm.n_tilde = (int)h[5];
    fmm.R = (int)h[6];
    const size_t nu = (size_t)fmm.m_tilde * fmm.k_tilde * fmm.R;
    const size_t nv = (size_t)fmm.k_tilde * fmm.n_tilde * fmm.R;
    const size_t nw = (size_t)fmm.m_tilde * fmm.n_tilde * fmm.R;
    fmm.U = (int*)malloc(sizeof(int) * nu);
    fmm.V = (int*)malloc(sizeof(int) * nv);
    fmm.W = (int*)malloc(sizeof(int) * nw);
    double* A = (double*)malloc(sizeof(double) * (size_t)(m * k + 1));
    double* B = (double*)malloc(sizeof(double) * (size_t)(k * n + 1));
    double* C = (double*)malloc(sizeof(double) * (size_t)(m * n + 1));
    if (!fmm.U || !fmm.V || !fmm.W || !A || !B || !C) { fprintf(stderr, "out of memory\n"); return 2; }
    if (!read_all(in, fmm.U, sizeof(int) * nu) || !read_all(in, fmm.V, sizeof(int) * nv) ||
        !read_all(in, fmm.W, sizeof(int) * nw) || !read_all(in, A, sizeof(double) * (size_t)(m * k)) ||
        !read_all(in, B, sizeof(double) * (size_t)(k * n)) || !read_all(in, C, sizeof(double) * (size_t)(m * n))) {
        fprintf(stderr, "short input\n");
        return 2;
    }
    fclose(in);

    bli_init();
    obj_t oA, oB, oC;
    bli_obj_create_with_attached_buffer(BLIS_DOUBLE, m, k, A, 1, m > 1 ? m : 1, &oA);
    bli_obj_create_with_attached_buffer(BLIS_DOUBLE, k, n, B, 1, k > 1 ? k : 1, &oB);
    bli_obj_create_with_attached_buffer(BLIS_DOUBLE, m, n, C, 1, m > 1 ? m : 1, &oC);
    double t0 = bl_clock();
    bli_strassen_ab_ex(&BLIS_ONE, &oA, &oB, &BLIS_ONE, &oC, fmm);
    double t = bl_clock() - t0;

    FILE* out = fopen(argv[2], "wb");
    if (!out) { perror(argv[2]); return 2; }
    if (fwrite(C, sizeof(double), (size_t)(m * n), out) != (size_t)(m * n)) { fprintf(stderr, "short write\n"); return 2; }
    fclose(out);
    printf("%.6f\n", t);
    free(fmm.U);
    free(fmm.V);
    free(fmm.W);
    free(A);
    free(B);
    free(C);
    bli_finalize();
    return 0;
}
