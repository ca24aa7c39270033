/*
 * Host-side coefficient algorithms: the reader of the U/V/W text files, the
 * built-in Strassen algorithm, the Brent-equation validator, the Kronecker
 * (two-level) generator and the wall clock.
 *
 * Follows frame/base/bli_read_fmm.c:24-86 (file format, fmm_t ownership),
 * frame/base/bli_strassen_ab.c:12-24 (STRASSEN_FMM) and
 * frame/util/bli_fmm_util.c:106-179 (bl_clock, CLOCK_MONOTONIC based).
 * Differences from the reference reader, all deliberate:
 *   - the header is read in the order the files are written, m~ k~ n~ R
 *     (232.txt has m~k~ = 6 rows of U); the reference stores it as m n k;
 *   - lines may be longer than 128 characters (444.txt rows are 146);
 *   - a missing file, a short file or a row with the wrong number of entries
 *     is reported instead of dereferencing NULL or reading garbage.
 */
#define _POSIX_C_SOURCE 200809L
#include "../../include/fmm_gb300.h"

#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static int strassen_u[4 * 7] = {1, 0, 1, 0, 1, -1, 0,  0, 0, 0, 0, 1, 0, 1,
                                0, 1, 0, 0, 0, 1, 0,   1, 1, 0, 1, 0, 0, -1};
static int strassen_v[4 * 7] = {1, 1, 0, -1, 0, 1, 0,  0, 0, 1, 0, 0, 1, 0,
                                0, 0, 0, 1, 0, 0, 1,   1, 0, -1, 0, 1, 0, 1};
static int strassen_w[4 * 7] = {1, 0, 0, 1, -1, 0, 1,  0, 0, 1, 0, 1, 0, 0,
                                0, 1, 0, 1, 0, 0, 0,   1, -1, 1, 0, 0, 1, 0};

fmm_t STRASSEN_FMM = {2, 2, 2, 7, strassen_u, strassen_v, strassen_w};

const char* fmm_status_string(int status)
{
    switch (status) {
    case FMM_OK: return "ok";
    case FMM_ERR_ARG: return "invalid argument";
    case FMM_ERR_FILE: return "coefficient file cannot be opened";
    case FMM_ERR_FORMAT: return "coefficient file malformed";
    case FMM_ERR_ALLOC: return "allocation failed";
    case FMM_ERR_CUDA: return "CUDA call failed";
    case FMM_ERR_UNSUPPORTED: return "unsupported size or option";
    case FMM_ERR_BRENT: return "coefficients violate the Brent equations";
    case FMM_ERR_DEVICE: return "kernel reported an error (bounded wait expired)";
    case FMM_ERR_WORKSPACE: return "workspace too small";
    case FMM_ERR_SCRATCH: return "problem exceeds the allocation-free entry point's static scratch";
    default: return "unknown status";
    }
}

/* Reads one whole line of any length into *buf (grown with realloc).
 * Returns the length, or -1 at end of file. */
static long read_line(FILE* fp, char** buf, size_t* cap)
{
    size_t len = 0;
    int c;
    if (*buf == NULL || *cap == 0) {
        *cap = 256;
        *buf = (char*)malloc(*cap);
        if (*buf == NULL) return -2;
    }
    while ((c = fgetc(fp)) != EOF) {
        if (len + 2 > *cap) {
            size_t ncap = *cap * 2;
            char* nb = (char*)realloc(*buf, ncap);
            if (nb == NULL) return -2;
            *buf = nb;
            *cap = ncap;
        }
        (*buf)[len++] = (char)c;
        if (c == '\n') break;
    }
    if (len == 0 && c == EOF) return -1;
    (*buf)[len] = '\0';
    return (long)len;
}

static int is_blank(const char* s)
{
    for (; *s; ++s)
        if (!isspace((unsigned char)*s)) return 0;
    return 1;
}

/* Parses up to `want` integers from `s` into out; returns how many were read
 * and sets *extra when more tokens follow. */
static int parse_ints(const char* s, int* out, int want, int* extra)
{
    int n = 0;
    char* end;
    *extra = 0;
    while (*s) {
        while (*s && isspace((unsigned char)*s)) ++s;
        if (!*s) break;
        long v = strtol(s, &end, 10);
        if (end == s) { *extra = 1; break; }
        if (n < want) out[n] = (int)v; else *extra = 1;
        ++n;
        s = end;
    }
    return n > want ? want : n;
}

int fmm_load(const char* file_name, fmm_t* out)
{
    if (out == NULL || file_name == NULL) return FMM_ERR_ARG;
    memset(out, 0, sizeof(*out));
    FILE* fp = fopen(file_name, "r");
    if (fp == NULL) return FMM_ERR_FILE;

    char* line = NULL;
    size_t cap = 0;
    long len;
    int hdr[4], extra = 0, got = 0, status = FMM_OK;

    /* header: first non-comment, non-blank line */
    while ((len = read_line(fp, &line, &cap)) >= 0) {
        if (line[0] == '#' || is_blank(line)) continue;
        got = parse_ints(line, hdr, 4, &extra);
        break;
    }
    if (len == -2) { status = FMM_ERR_ALLOC; goto done; }
    if (got != 4 || hdr[0] <= 0 || hdr[1] <= 0 || hdr[2] <= 0 || hdr[3] <= 0) {
        status = FMM_ERR_FORMAT;
        goto done;
    }
    {
        int mt = hdr[0], kt = hdr[1], nt = hdr[2], R = hdr[3];
        int aparts = mt * kt, bparts = kt * nt, cparts = mt * nt;
        int total = aparts + bparts + cparts, row = 0;
        int* U = (int*)calloc((size_t)aparts * R, sizeof(int));
        int* V = (int*)calloc((size_t)bparts * R, sizeof(int));
        int* W = (int*)calloc((size_t)cparts * R, sizeof(int));
        if (!U || !V || !W) {
            free(U); free(V); free(W);
            status = FMM_ERR_ALLOC;
            goto done;
        }
        while (row < total && (len = read_line(fp, &line, &cap)) >= 0) {
            if (line[0] == '#' || is_blank(line)) continue;
            int* dst;
            if (row < aparts) dst = U + (size_t)row * R;
            else if (row < aparts + bparts) dst = V + (size_t)(row - aparts) * R;
            else dst = W + (size_t)(row - aparts - bparts) * R;
            if (parse_ints(line, dst, R, &extra) != R || extra) {
                status = FMM_ERR_FORMAT;
                break;
            }
            ++row;
        }
        if (status == FMM_OK && row != total) status = FMM_ERR_FORMAT;
        if (status != FMM_OK) {
            free(U); free(V); free(W);
            goto done;
        }
        out->m_tilde = mt;
        out->k_tilde = kt;
        out->n_tilde = nt;
        out->R = R;
        out->U = U;
        out->V = V;
        out->W = W;
    }
done:
    free(line);
    fclose(fp);
    return status;
}

fmm_t new_fmm(const char* file_name)
{
    fmm_t f;
    if (fmm_load(file_name, &f) != FMM_OK) memset(&f, 0, sizeof(f));
    return f;
}

void free_fmm(fmm_t fmm)
{
    if (fmm.U == STRASSEN_FMM.U) return; /* never free the built-in tables */
    free(fmm.U);
    free(fmm.V);
    free(fmm.W);
}

int fmm_copy(const fmm_t* src, fmm_t* dst)
{
    if (!src || !dst || src->R <= 0) return FMM_ERR_ARG;
    size_t a = (size_t)src->m_tilde * src->k_tilde * src->R;
    size_t b = (size_t)src->k_tilde * src->n_tilde * src->R;
    size_t c = (size_t)src->m_tilde * src->n_tilde * src->R;
    fmm_t o = *src;
    o.U = (int*)malloc(a * sizeof(int));
    o.V = (int*)malloc(b * sizeof(int));
    o.W = (int*)malloc(c * sizeof(int));
    if (!o.U || !o.V || !o.W) {
        free(o.U); free(o.V); free(o.W);
        return FMM_ERR_ALLOC;
    }
    memcpy(o.U, src->U, a * sizeof(int));
    memcpy(o.V, src->V, b * sizeof(int));
    memcpy(o.W, src->W, c * sizeof(int));
    *dst = o;
    return FMM_OK;
}

/* Counts the violated Brent equations: A block (a,b) x B block (b2,c) must
 * reach C block (a2,c2) with total weight sum_r U[(a,b),r] V[(b2,c),r]
 * W[(a2,c2),r] = [a==a2][b==b2][c==c2]. The sums are accumulated from the
 * nonzero coefficients of each product (sum_r nnzU*nnzV*nnzW terms) into one
 * counter per equation, so two-level algorithms (16.7 M equations, 9 M terms
 * for 444 x 444) check in milliseconds; past 2^26 equations it falls back to
 * one dot product per equation. */
static long brent_direct(const fmm_t* f)
{
    const int mt = f->m_tilde, kt = f->k_tilde, nt = f->n_tilde, R = f->R;
    long bad = 0;
    for (int a = 0; a < mt; ++a)
    for (int b = 0; b < kt; ++b)
    for (int b2 = 0; b2 < kt; ++b2)
    for (int c = 0; c < nt; ++c)
    for (int a2 = 0; a2 < mt; ++a2)
    for (int c2 = 0; c2 < nt; ++c2) {
        const int* u = f->U + (size_t)(a * kt + b) * R;
        const int* v = f->V + (size_t)(b2 * nt + c) * R;
        const int* w = f->W + (size_t)(a2 * nt + c2) * R;
        long sum = 0;
        for (int r = 0; r < R; ++r) sum += (long)u[r] * v[r] * w[r];
        long want = (a == a2 && b == b2 && c == c2) ? 1 : 0;
        if (sum != want) ++bad;
    }
    return bad;
}

int fmm_check_brent(const fmm_t* f, long* n_bad)
{
    if (!f || f->R <= 0 || !f->U || !f->V || !f->W) return FMM_ERR_ARG;
    const int mt = f->m_tilde, kt = f->k_tilde, nt = f->n_tilde, R = f->R;
    if (mt <= 0 || kt <= 0 || nt <= 0) return FMM_ERR_ARG;
    const size_t na = (size_t)mt * kt, nb = (size_t)kt * nt, nc = (size_t)mt * nt;
    const size_t neq = na * nb * nc;
    long bad = -1;
    int64_t* acc = neq <= ((size_t)1 << 26) ? (int64_t*)calloc(neq, sizeof(int64_t)) : NULL;
    int* iu = acc ? (int*)malloc(sizeof(int) * na) : NULL;
    int* iv = acc ? (int*)malloc(sizeof(int) * nb) : NULL;
    int* iw = acc ? (int*)malloc(sizeof(int) * nc) : NULL;
    if (acc && iu && iv && iw) {
        for (int r = 0; r < R; ++r) {
            int cu = 0, cv = 0, cw = 0;
            for (size_t q = 0; q < na; ++q) if (f->U[q * R + r]) iu[cu++] = (int)q;
            for (size_t q = 0; q < nb; ++q) if (f->V[q * R + r]) iv[cv++] = (int)q;
            for (size_t q = 0; q < nc; ++q) if (f->W[q * R + r]) iw[cw++] = (int)q;
            for (int x = 0; x < cu; ++x)
                for (int y = 0; y < cv; ++y) {
                    const int64_t uv = (int64_t)f->U[(size_t)iu[x] * R + r] * f->V[(size_t)iv[y] * R + r];
                    int64_t* row = acc + ((size_t)iu[x] * nb + (size_t)iv[y]) * nc;
                    for (int z = 0; z < cw; ++z) row[iw[z]] += uv * f->W[(size_t)iw[z] * R + r];
                }
        }
        bad = 0;
        for (int a = 0; a < mt; ++a)
        for (int b = 0; b < kt; ++b)
        for (int b2 = 0; b2 < kt; ++b2)
        for (int c = 0; c < nt; ++c) {
            const int64_t* row = acc + ((size_t)(a * kt + b) * nb + (size_t)(b2 * nt + c)) * nc;
            for (int a2 = 0; a2 < mt; ++a2)
                for (int c2 = 0; c2 < nt; ++c2) {
                    const int64_t want = (a == a2 && b == b2 && c == c2) ? 1 : 0;
                    if (row[a2 * nt + c2] != want) ++bad;
                }
        }
    }
    free(acc);
    free(iu);
    free(iv);
    free(iw);
    if (bad < 0) bad = brent_direct(f);
    if (n_bad) *n_bad = bad;
    return bad ? FMM_ERR_BRENT : FMM_OK;
}

/* Row q of a factor for an (rows_t x cols_t) block grid of the flat
 * algorithm, built from the outer block (q_o) and inner block (q_i). */
static void kron_factor(const int* fo, int ro_t, int co_t, int Ro,
                        const int* fi, int ri_t, int ci_t, int Ri, int* out)
{
    const int rows = ro_t * ri_t, cols = co_t * ci_t, R = Ro * Ri;
    for (int a = 0; a < rows; ++a)
    for (int b = 0; b < cols; ++b) {
        int qo = (a / ri_t) * co_t + (b / ci_t);
        int qi = (a % ri_t) * ci_t + (b % ci_t);
        int* dst = out + (size_t)(a * cols + b) * R;
        for (int r1 = 0; r1 < Ro; ++r1)
            for (int r2 = 0; r2 < Ri; ++r2)
                dst[r1 * Ri + r2] = fo[(size_t)qo * Ro + r1] * fi[(size_t)qi * Ri + r2];
    }
}

int fmm_kron(const fmm_t* o, const fmm_t* i, fmm_t* out)
{
    if (!o || !i || !out || o->R <= 0 || i->R <= 0) return FMM_ERR_ARG;
    fmm_t f;
    f.m_tilde = o->m_tilde * i->m_tilde;
    f.k_tilde = o->k_tilde * i->k_tilde;
    f.n_tilde = o->n_tilde * i->n_tilde;
    f.R = o->R * i->R;
    f.U = (int*)malloc(sizeof(int) * (size_t)f.m_tilde * f.k_tilde * f.R);
    f.V = (int*)malloc(sizeof(int) * (size_t)f.k_tilde * f.n_tilde * f.R);
    f.W = (int*)malloc(sizeof(int) * (size_t)f.m_tilde * f.n_tilde * f.R);
    if (!f.U || !f.V || !f.W) {
        free(f.U); free(f.V); free(f.W);
        return FMM_ERR_ALLOC;
    }
    kron_factor(o->U, o->m_tilde, o->k_tilde, o->R, i->U, i->m_tilde, i->k_tilde, i->R, f.U);
    kron_factor(o->V, o->k_tilde, o->n_tilde, o->R, i->V, i->k_tilde, i->n_tilde, i->R, f.V);
    kron_factor(o->W, o->m_tilde, o->n_tilde, o->R, i->W, i->m_tilde, i->n_tilde, i->R, f.W);
    *out = f;
    return FMM_OK;
}

static double clock_origin = 0.0;

double bl_clock(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    if (clock_origin == 0.0) clock_origin = (double)ts.tv_sec;
    return ((double)ts.tv_sec - clock_origin) + ts.tv_nsec * 1.0e-9;
}
