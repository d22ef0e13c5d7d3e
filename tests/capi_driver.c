/*
 * capi_driver.c -- a plain C11 caller of the library through include/bs2e.h,
 * compiled with the host C compiler (gcc) against libbs2e.so.  It stands in
 * for the Fortran shim of basis_setup (main_basis_setup.f90:77-116): the
 * calls, their order and the two-phase count/fill pattern are the ones the
 * shim makes, and the compiler checks every declaration it uses against the
 * header while the linker resolves each entry point in the library.
 *
 * Usage: capi_driver <input> <output>
 *   input  (little-endian): int64 k, k_GL, max_k, n_knots, n_config, L, full,
 *          Z, n_l, cap_order; double cap_r0, cap_eta_re, cap_eta_im;
 *          double knots[n_knots]; int64 configs[5 * n_config] (n1 n2 l1 l2 eqv)
 *   output: int64 status, nnz_H, nnz_S, n_b, nnz4, nnz6;
 *          H: int64 index_ptr[n_config+1], int64 indices[nnz_H], double data[2*nnz_H];
 *          S: likewise with nnz_S;
 *          double R[(max_k+1)] of key (1, 1, 1, 1), then of key (2, 3, 1, 4)
 * Exit status 0 when every call returned BS2E_OK; otherwise the failing
 * call's message goes to stderr.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "bs2e.h"

static int fail(bs2e_handle *h, const char *what, bs2e_status st) {
    char msg[512] = "";
    if (h) bs2e_last_error(h, msg, (int64_t)sizeof msg);
    fprintf(stderr, "%s failed: status %d: %s\n", what, (int)st, msg);
    return 1;
}

#define CALL(h, x)                                   \
    do {                                             \
        bs2e_status st_ = (x);                       \
        if (st_ != BS2E_OK) return fail(h, #x, st_); \
    } while (0)

static int rd(FILE *f, void *p, size_t n) { return fread(p, 1, n, f) == n ? 0 : 1; }
static int wr(FILE *f, const void *p, size_t n) { return fwrite(p, 1, n, f) == n ? 0 : 1; }

int main(int argc, char **argv) {
    if (argc != 3) {
        fprintf(stderr, "usage: %s <input> <output>\n", argv[0]);
        return 2;
    }
    FILE *in = fopen(argv[1], "rb");
    if (!in) return 2;
    int64_t hdr[10];
    double cap[3];
    if (rd(in, hdr, sizeof hdr) || rd(in, cap, sizeof cap)) return 2;
    const int64_t k = hdr[0], k_GL = hdr[1], max_k = hdr[2], n_knots = hdr[3],
                  n_config = hdr[4], L = hdr[5], full = hdr[6], Z = hdr[7], n_l = hdr[8],
                  cap_order = hdr[9];
    double *knots = malloc(sizeof(double) * (size_t)n_knots);
    bs2e_config *cf = malloc(sizeof(bs2e_config) * (size_t)(n_config > 0 ? n_config : 1));
    if (!knots || !cf || rd(in, knots, sizeof(double) * (size_t)n_knots) ||
        rd(in, cf, sizeof(bs2e_config) * (size_t)n_config))
        return 2;
    fclose(in);

    bs2e_opts opts;
    bs2e_default_opts(&opts);
    opts.precision = BS2E_PREC_FP64;
    bs2e_handle *h = NULL;
    CALL(NULL, bs2e_create(knots, n_knots, k, k_GL, max_k, &opts, &h));
    int64_t n_b = 0, n_iv = 0, nnz4 = 0, nnz6 = 0;
    CALL(h, bs2e_sizes(h, &n_b, &n_iv, &nnz4, &nnz6));
    CALL(h, bs2e_slater(h));                   /* setup_Slater_integrals */
    CALL(h, bs2e_rk(h, 0, max_k + 1));         /* compute_R_k_map */
    CALL(h, bs2e_one_body(h, Z, n_l, cap_order, cap[0], cap[1], cap[2], NULL, NULL));
    int64_t nnz_H = 0, nnz_S = 0;
    CALL(h, bs2e_block_count(h, cf, n_config, L, full, &nnz_H, &nnz_S)); /* count_nnz */
    int64_t *Hp = malloc(sizeof(int64_t) * (size_t)(n_config + 1));
    int64_t *Sp = malloc(sizeof(int64_t) * (size_t)(n_config + 1));
    int64_t *Hi = malloc(sizeof(int64_t) * (size_t)(nnz_H > 0 ? nnz_H : 1));
    int64_t *Si = malloc(sizeof(int64_t) * (size_t)(nnz_S > 0 ? nnz_S : 1));
    double *Hd = malloc(sizeof(double) * 2 * (size_t)(nnz_H > 0 ? nnz_H : 1));
    double *Sd = malloc(sizeof(double) * 2 * (size_t)(nnz_S > 0 ? nnz_S : 1));
    if (!Hp || !Sp || !Hi || !Si || !Hd || !Sd) return 2;
    /* construct_block_tensor into caller-allocated arrays (one-body set above) */
    CALL(h, bs2e_block_fill(h, cf, n_config, L, full, NULL, 0, NULL, Hp, Hi, Hd, Sp, Si, Sd));
    const int64_t keys[2][4] = {{1, 1, 1, 1}, {2, 3, 1, 4}};
    double *rk = malloc(sizeof(double) * (size_t)(max_k + 1) * 2);
    if (!rk) return 2;
    CALL(h, bs2e_rk_get(h, keys[0], rk));
    CALL(h, bs2e_rk_get(h, keys[1], rk + max_k + 1));
    CALL(h, bs2e_destroy(h));

    FILE *out = fopen(argv[2], "wb");
    if (!out) return 2;
    const int64_t head[6] = {0, nnz_H, nnz_S, n_b, nnz4, nnz6};
    if (wr(out, head, sizeof head) || wr(out, Hp, sizeof(int64_t) * (size_t)(n_config + 1)) ||
        wr(out, Hi, sizeof(int64_t) * (size_t)nnz_H) ||
        wr(out, Hd, sizeof(double) * 2 * (size_t)nnz_H) ||
        wr(out, Sp, sizeof(int64_t) * (size_t)(n_config + 1)) ||
        wr(out, Si, sizeof(int64_t) * (size_t)nnz_S) ||
        wr(out, Sd, sizeof(double) * 2 * (size_t)nnz_S) ||
        wr(out, rk, sizeof(double) * (size_t)(max_k + 1) * 2))
        return 2;
    fclose(out);
    free(knots);
    free(cf);
    free(Hp);
    free(Sp);
    free(Hi);
    free(Si);
    free(Hd);
    free(Sd);
    free(rk);
    return 0;
}
