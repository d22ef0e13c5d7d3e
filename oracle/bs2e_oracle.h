/*
 * bs2e_oracle.h -- CPU oracle for the two-electron matrix-element path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * Fortran (edvinolo/b-spline-two-e, src/mat_els + src/tools) that the parity
 * tests compare the GPU library with, and the timed CPU baseline.  Only tests/, the smoke check
 * and the CPU-baseline leg of bench.py may load it.  The GPU library never
 * links or calls anything here.
 *
 * Conventions follow the reference: all integers int64 (the reference builds
 * with -fdefault-integer-8), Fortran (1-based) basis / interval indices in
 * every exported index array, column-major 2-D arrays, complex128 values as
 * interleaved (re, im) doubles.
 */
#ifndef BS2E_ORACLE_H
#define BS2E_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One two-electron configuration, as type(config) in src/tools/orbital_tools.f90:15-19. */
typedef struct {
    int64_t n1, n2; /* radial B-spline indices (1-based, basis numbering) */
    int64_t l1, l2; /* orbital angular momenta, l1 >= l2 */
    int64_t eqv;    /* 1 if (n1,l1) == (n2,l2) */
} or_config;

/* Gauss-Legendre nodes/weights on [-1,1] (src/tools/quad_tools.f90:14-27). */
void or_gauss_legendre(int64_t q, double *x, double *w);

/* de Boor value (ideriv=0) or derivative of the single B-spline with full
 * index jspline (1-based) at x, interval hint iv (1-based breakpoint interval),
 * as BVALUE_D with a unit coefficient vector (src/tools/bspline_tools.f90:151-224). */
double or_bvalue(const double *t, int64_t n, int64_t k, double x, int64_t ideriv,
                 int64_t iv, int64_t jspline);

/* Angular algebra (src/tools/wigner_tools.f90). Arguments are plain (not doubled) integers. */
double or_three_j(int64_t ja, int64_t jb, int64_t jc, int64_t ma, int64_t mb, int64_t mc);
double or_six_j(int64_t ja, int64_t jb, int64_t jc, int64_t jd, int64_t je, int64_t jf);
double or_C_red_mat(int64_t k, int64_t a, int64_t b);
double or_ang_k_LS(int64_t k, int64_t la, int64_t lb, int64_t lc, int64_t ld, int64_t L);

/* COO sizes of the primitives (src/tools/sparse_array_tools.f90:276-324). */
int64_t or_nnz4(int64_t n_knots, int64_t k);
int64_t or_nnz6(int64_t n_knots, int64_t k);

/* Slater primitives (src/mat_els/mat_els.f90:172-292, 392-491).
 * rk, rmk: nnz4 x (max_k+1) column-major; idx4: 3 x nnz4 (iv, i, j) column-major.
 * rdk: nnz6 x (max_k+1); idx6: 5 x nnz6 (iv, i, i_p, j, j_p).
 * nthreads <= 0 means "all OpenMP threads". */
void or_slater(const double *knots, int64_t n_knots, int64_t k, int64_t k_GL, int64_t max_k,
               double *rk, double *rmk, int64_t *idx4, double *rdk, int64_t *idx6, int nthreads);

/* R^k map (src/tools/sparse_array_tools.f90:452-493).  Keys [a,b,c,d] (1-based)
 * with |a-c|<k, |b-d|<k are stored banded: element (a,b,c,d,kk) at
 *   ((((a-1)*N + (b-1))*W + (c-a+k-1))*W + (d-b+k-1))*(max_k+1) + kk,  W = 2k-1.
 * R must hold N*N*W*W*(max_k+1) doubles; it is zeroed here. */
void or_rk_map(int64_t n_b, int64_t k, int64_t max_k, int64_t nnz4, const double *rk,
               const double *rmk, const int64_t *idx4, int64_t nnz6, const double *rdk,
               const int64_t *idx6, double *R);

/* R^k of whole tiles (a, b) for bases too large for or_slater + or_rk_map:
 * out[t][dc][dd][kk] = R^k[a, b, a+dc-(k-1), b+dd-(k-1)] for tile t = (ab[2t],
 * ab[2t+1]) (1-based), W = 2k-1 values of dc and dd, zero where c or d falls
 * outside 1..n_b.  The primitives a key needs are computed with or_slater's
 * arithmetic (compute_Slater_off_diag / compute_Slater_diag,
 * mat_els.f90:392-491), spline values cached per interval, and added in the
 * order compute_R_K_map (sparse_array_tools.f90:452-493) adds them into that
 * key, so each value equals or_rk_map's bit for bit.  OpenMP over tiles. */
void or_rk_tiles(const double *knots, int64_t n_knots, int64_t k, int64_t k_GL, int64_t max_k,
                 int64_t n_tiles, const int64_t *ab, double *out, int nthreads);

/* Configuration list of one symmetry block (src/tools/orbital_tools.f90:119-216).
 * spin = 0 is the reference (singlet); spin = 1 gives the triplet list.
 * Returns the count; writes the list when out != NULL. */
int64_t or_count_configs(int64_t L, int64_t parity_odd, int64_t max_l_1p, int64_t n_b,
                         int64_t k, int64_t max_n_b, int64_t n_all_l, int64_t l2_max,
                         int64_t spin, or_config *out);

/* count_nnz (src/mat_els/hamiltonian.f90:348-416); writes nnz[0]=H, nnz[1]=S. */
void or_count_nnz(const or_config *cf, int64_t n_config, int64_t L, int64_t spin, int64_t k,
                  int64_t max_k, int64_t full, int64_t *nnz);

/* construct_block_tensor (src/mat_els/hamiltonian.f90:106-283) for rows
 * [row_begin, row_end) (0-based half-open).  CSR pointers are 1-based and local
 * to the row range (first entry 1).  Pass NULL output arrays to count only; the
 * counts are returned in nnz_out[0]=H, nnz_out[1]=S.  H_scale (may be NULL)
 * receives, per H entry, the sum of the magnitudes of every term added into it,
 * which normalises rounding differences of a cancelling sum.
 * H1p: n_b x n_b x n_l complex column-major (one block per l); S: n_b x n_b. */
void or_construct_block(const or_config *cf, int64_t n_config, int64_t L, int64_t spin,
                        int64_t k, int64_t n_b, int64_t max_k, int64_t full, const double *R,
                        const double *H1p, int64_t n_l, const double *S, int64_t row_begin,
                        int64_t row_end, int64_t *H_ptr, int64_t *H_idx, double *H_data,
                        double *H_scale, int64_t *S_ptr, int64_t *S_idx, double *S_data,
                        int64_t *nnz_out);

/* or_construct_block with R given as tiles (or_rk_tiles layout): the R^k
 * values of row (n_a, n_b) are read from tile tile_of[(n_a-1)*n_b_total +
 * (n_b-1)] of R (each row reads only its own tile).  A row whose tile is
 * missing (index < 0) stops the assembly with nnz_out[0] = -1. */
void or_construct_block_tiles(const or_config *cf, int64_t n_config, int64_t L, int64_t spin,
                              int64_t k, int64_t n_b, int64_t max_k, int64_t full,
                              const double *R, const int64_t *tile_of, const double *H1p,
                              int64_t n_l, const double *S, int64_t row_begin, int64_t row_end,
                              int64_t *H_ptr, int64_t *H_idx, double *H_data, double *H_scale,
                              int64_t *S_ptr, int64_t *S_idx, double *S_data, int64_t *nnz_out);

/* One-body matrices (src/mat_els/mat_els.f90:47-118, 294-346): S and
 * H_l = -1/2 d2/dr2 + l(l+1)/(2r^2) - Z/r + CAP, complex n_b x n_b column-major. */
void or_setup_S(const double *knots, int64_t n_knots, int64_t k, int64_t k_GL, double *S);
void or_setup_H1p(const double *knots, int64_t n_knots, int64_t k, int64_t k_GL, int64_t Z,
                  int64_t l, int64_t cap_order, double cap_r0, double cap_eta_re,
                  double cap_eta_im, double *H);

/* setup_radial_dip (src/mat_els/mat_els.f90:120-170, 348-390): gauge 0 = length
 * ('l': r_mat), 1 = velocity ('v': dr_mat, r_inv_mat).  Complex n_b x n_b
 * column-major; unused outputs may be NULL. */
void or_setup_radial_dip(const double *knots, int64_t n_knots, int64_t k, int64_t k_GL,
                         int64_t gauge, double *r_mat, double *dr_mat, double *r_inv_mat);

/* construct_dip_block_tensor with init_dip_block (src/mat_els/dipole.f90:8-47,
 * 87-146) for the block (row symmetry (L1, M1, pi1), column symmetry (L2, M2,
 * pi2)) and polarisation q; compute = 0 gives the empty block as the reference
 * does for skipped pairs.  Pass NULL outputs to count only (nnz returned). */
int64_t or_dip_block(const or_config *rows, int64_t n_rows, int64_t L1, int64_t M1, int64_t pi1,
                     const or_config *cols, int64_t n_cols, int64_t L2, int64_t M2, int64_t pi2,
                     int64_t q, int64_t compute, int64_t k, int64_t n_b, int64_t gauge,
                     const double *S, const double *r_mat, const double *dr_mat,
                     const double *r_inv_mat, int64_t *ptr, int64_t *idx, double *data);

/* Sparse products of a 1-based CSR matrix with a complex vector
 * (src/tools/sparse_array_tools.f90:966-1074): op 0 = CSR_mv (y = A x),
 * op 1 = CSR_T_mv (y = A^T x, no conjugation), op 2 = CSR_mv_sym, i.e.
 * mkl_zcsrsymv('U'): A complex symmetric, only entries with column >= row
 * used.  data, x, y complex128 interleaved; scale (optional) receives
 * sum |a_ij| |x_j| per output entry. */
void or_csr_mv(int64_t op, int64_t n_rows, int64_t n_cols, const int64_t *ptr,
               const int64_t *idx, const double *data, const double *x, double *y,
               double *scale);

/* CSR_from_block (src/tools/block_tools.f90:188-234): block (i, j) of the
 * n_rb x n_cb block matrix is b = i + n_rb*j; rows of block row i from block
 * (i, 0); arrays of empty blocks are not read.  out_ptr has sum(rows) + 1
 * entries; returns the number of entries written. */
int64_t or_csr_from_blocks(int64_t n_rb, int64_t n_cb, const int64_t *shapes, const int64_t *nnz,
                           const int64_t *const *ptr, const int64_t *const *idx,
                           const double *const *data, int64_t *out_ptr, int64_t *out_idx,
                           double *out_data);

#ifdef __cplusplus
}
#endif
#endif
