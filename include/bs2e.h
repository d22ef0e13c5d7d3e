/*
 * bs2e.h -- C ABI of the GB300 two-electron matrix-element library.
 *
 * Drop-in for the two-electron path that basis_setup runs in
 * edvinolo/b-spline-two-e (src/apps/main_basis_setup.f90:77-85 and :105-116):
 * radial Slater-integral primitives, the R^k[a,b,c,d] store, the 3j/6j
 * angular weights and the sparse CSR assembly of every symmetry block of the
 * two-electron Hamiltonian H and overlap S.  The Fortran host binds these
 * entry points through ISO_C_BINDING; nothing here uses C++ or torch types.
 *
 * Conventions (all follow the reference, which is built with
 * -fdefault-integer-8):
 *   - every integer is int64_t; basis, interval and configuration indices are
 *     1-based (Fortran numbering) wherever they cross this boundary;
 *   - 2-D arrays are column-major;
 *   - "complex" arrays are complex128 stored as interleaved (re, im) doubles,
 *     i.e. Fortran complex(c_double_complex);
 *   - CSR output is the reference's CSR_matrix layout
 *     (src/tools/sparse_array_tools.f90:63-135): index_ptr(rows+1) and
 *     indices(nnz) 1-based, columns ascending within a row, data complex128.
 *
 * Every call returns a bs2e_status; BS2E_OK is 0.  On error the handle keeps
 * a message readable with bs2e_last_error().  Calls on one handle are
 * serialised by an internal mutex, so a Fortran OpenMP loop may call the
 * block entry points concurrently (as main_basis_setup.f90:105 does).
 */
#ifndef BS2E_H
#define BS2E_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define BS2E_API __attribute__((visibility("default")))
#else
#define BS2E_API
#endif

typedef int32_t bs2e_status;

enum {
    BS2E_OK = 0,
    BS2E_ERR_ARG = 1,     /* invalid argument (sizes, knots, ranges) */
    BS2E_ERR_NOMEM = 2,   /* device or host allocation failed */
    BS2E_ERR_CUDA = 3,    /* CUDA runtime error */
    BS2E_ERR_COUNT = 4,   /* count/fill disagreement (reference count_nnz contract broken) */
    BS2E_ERR_TIMEOUT = 5, /* a bounded device wait gave up */
    BS2E_ERR_STATE = 6,   /* call made out of order (e.g. fill before bs2e_rk) */
    BS2E_ERR_NODEV = 7,   /* no CUDA device available */
    BS2E_ERR_ORDER = 8    /* configuration list is not in basis order */
};

/* Arithmetic used for the R^k store and the sum over multipoles. */
enum {
    BS2E_PREC_FP64 = 0,  /* plain path: every operation in FP64 */
    BS2E_PREC_MIXED = 1  /* R^k stored as scaled FP32 pairs, k-sum in FP32-pair arithmetic */
};

typedef struct bs2e_handle bs2e_handle;

typedef struct {
    int64_t precision; /* BS2E_PREC_FP64 (default) or BS2E_PREC_MIXED */
    int64_t device;    /* CUDA device ordinal (default 0) */
    int64_t stage_bytes; /* size of each of the two HBM staging areas of fills
                            into host arrays (0 = 8 GiB) */
    int64_t reserved[5];
} bs2e_opts;

/* One two-electron configuration: type(config) of src/tools/orbital_tools.f90:15-19
 * as a bind(C) record (n(2), l(2), eqv as int64). */
typedef struct {
    int64_t n1, n2;
    int64_t l1, l2;
    int64_t eqv;
} bs2e_config;

/* Fills *opts with defaults (FP64, device 0). */
BS2E_API void bs2e_default_opts(bs2e_opts *opts);

/* Creates a handle for one B-spline basis.  Replaces splines%init(k,grid)
 * (src/tools/bspline_tools.f90:27-40) together with the r_k/r_m_k/r_d_k%init
 * calls of main_basis_setup.f90:77-79: knots is the full knot vector t(1:n+k),
 * n_b = n-2 splines are kept (first and last dropped), k_GL Gauss-Legendre
 * points per breakpoint interval, multipoles k = 0..max_k. */
BS2E_API bs2e_status bs2e_create(const double *knots, int64_t n_knots, int64_t k, int64_t k_GL,
                                 int64_t max_k, const bs2e_opts *opts, bs2e_handle **out);

BS2E_API bs2e_status bs2e_destroy(bs2e_handle *h);

/* Copies the last error message (NUL-terminated, truncated to len). */
BS2E_API bs2e_status bs2e_last_error(const bs2e_handle *h, char *buf, int64_t len);

/* Basis size n_b, interval count and the COO sizes nnz4/nnz6 of the
 * reference's sparse_4d / sparse_6d primitives (sparse_array_tools.f90:276-324). */
BS2E_API bs2e_status bs2e_sizes(const bs2e_handle *h, int64_t *n_b, int64_t *n_iv, int64_t *nnz4,
                                int64_t *nnz6);

/* Slater primitives on the device.  Replaces setup_Slater_integrals
 * (src/mat_els/mat_els.f90:172-292): per-interval moments r_k, r_m_k and the
 * same-interval kink-split 2-D integrals r_d_k for k = 0..max_k. */
BS2E_API bs2e_status bs2e_slater(bs2e_handle *h);

/* Copies the primitives out in the reference's COO order (for parity checks):
 * r_k, r_m_k: nnz4 x (max_k+1); idx4: 3 x nnz4 = (iv, i, j);
 * r_d_k: nnz6 x (max_k+1); idx6: 5 x nnz6 = (iv, i, i_p, j, j_p).
 * Any pointer may be NULL to skip that array. */
BS2E_API bs2e_status bs2e_get_primitives(bs2e_handle *h, double *r_k, double *r_m_k,
                                         int64_t *idx4, double *r_d_k, int64_t *idx6);

/* Builds the R^k store for multipoles k_first .. k_first+k_count-1 (pass 0 and
 * max_k+1 for all).  Replaces compute_R_k_map (src/tools/sparse_array_tools.f90:452-493). */
BS2E_API bs2e_status bs2e_rk(bs2e_handle *h, int64_t k_first, int64_t k_count);

/* R^k values of one key [a,b,c,d] (1-based, |a-c|<k, |b-d|<k) for k = 0..max_k,
 * as Nd_DOK%get_val (src/tools/sparse_array_tools.f90:536-555). */
BS2E_API bs2e_status bs2e_rk_get(bs2e_handle *h, const int64_t key[4], double *vals);

/* Batched bs2e_rk_get: keys is 4 x n column-major, vals is (max_k+1) x n. */
BS2E_API bs2e_status bs2e_rk_get_batch(bs2e_handle *h, int64_t n, const int64_t *keys,
                                       double *vals);

/* Multipole k of the whole R^k store as doubles, out[a][b][c-a+k_o-1][d-b+k_o-1]
 * (C order, N*N*W*W values, W = 2*k_o-1, k_o the spline order, 0-based a, b;
 * zero where c or d falls outside the basis).  The mixed store is returned as
 * the exact double value of its scaled FP32 pair.  on_device = 1: out is a
 * device pointer.  For dumps and precision studies; Nd_DOK offers only
 * get_val (sparse_array_tools.f90:536-555). */
BS2E_API bs2e_status bs2e_rk_export(bs2e_handle *h, int64_t k, double *out, int64_t on_device);

/* bs2e_rk_get_batch without any device allocation.  This entry point has no
 * counterpart in the reference.  It is for callers that can't allocate device
 * memory at lookup time: a caller that has filled HBM with CSR blocks can't
 * risk an allocation failing, and the cudaFree of the allocating lookup waits
 * for the whole device, stalling work on other streams.  Keys and values are
 * staged in one file-scope device array of at most 4096 keys (1.125 MiB on
 * every GPU that loads the library, held until the process exits); larger n
 * is rejected with BS2E_ERR_ARG.  bs2e_create reserves the array on the
 * handle's device (it looks up the array's address with cudaGetSymbolAddress
 * and loads the lookup kernel), so the array is resident before the caller
 * fills HBM; if that set-up is missing for a device, the first call on it
 * (n = 0 included) does it and should come before any stream capture there.
 * The address holds for the device's current primary context; a handle does
 * not survive cudaDeviceReset.  Allocation failures during set-up return
 * BS2E_ERR_NOMEM.  All calls on a device share the array, which keeps the
 * last call's contents; calls whose GPU work overlaps race on it. */
BS2E_API bs2e_status bs2e_rk_get_batch_static(bs2e_handle *h, int64_t n, const int64_t *keys,
                                              double *vals);

/* Uploads the one-body matrices used by every block: H1p is n_b x n_b x n_l
 * complex (H_vec(l)%data for l = 0..n_l-1, main_basis_setup.f90:95-99), S is
 * n_b x n_b complex (main_basis_setup.f90:91-93). */
BS2E_API bs2e_status bs2e_set_one_body(bs2e_handle *h, const double *H1p, int64_t n_l,
                                       const double *S);

/* Computes the one-body matrices on the device instead (setup_S and
 * setup_H_one_particle, src/mat_els/mat_els.f90:47-118, hydrogenic potential
 * potentials.f90:35-43 and the CAP of CAP_tools.f90:23-33), keeps them for the
 * blocks and optionally copies them out (H1p / S may be NULL). */
BS2E_API bs2e_status bs2e_one_body(bs2e_handle *h, int64_t Z, int64_t n_l, int64_t cap_order,
                                   double cap_r0, double cap_eta_re, double cap_eta_im,
                                   double *H1p, double *S);

/* Number of non-zeros of the H and S blocks of one symmetry (L, singlet).
 * Same contract as count_nnz (src/mat_els/hamiltonian.f90:348-416): the counts
 * size the CSR arrays that bs2e_block_fill writes.  full = 1 gives the whole
 * block, full = 0 the upper triangle (hamiltonian.f90:131-135). */
BS2E_API bs2e_status bs2e_block_count(bs2e_handle *h, const bs2e_config *configs,
                                      int64_t n_config, int64_t L, int64_t full, int64_t *nnz_H,
                                      int64_t *nnz_S);

/* Fills one symmetry block into caller-allocated host arrays sized by
 * bs2e_block_count.  Replaces construct_block_tensor
 * (src/mat_els/hamiltonian.f90:106-283).  H1p / S may be NULL to use the
 * matrices set by bs2e_set_one_body / bs2e_one_body. */
BS2E_API bs2e_status bs2e_block_fill(bs2e_handle *h, const bs2e_config *configs,
                                     int64_t n_config, int64_t L, int64_t full, const double *H1p,
                                     int64_t n_l, const double *S, int64_t *H_index_ptr,
                                     int64_t *H_indices, double *H_data, int64_t *S_index_ptr,
                                     int64_t *S_indices, double *S_data);

/* Extended forms.  spin = 0 is the reference's singlet coupling; spin = 1
 * builds the triplet block (exchange terms change sign; equivalent
 * configurations belong to odd L), which the reference does not have.
 * out_on_device = 1 means the six output pointers are CUDA device pointers
 * (inputs already resident in HBM); 0 means host memory. */
BS2E_API bs2e_status bs2e_block_count_ex(bs2e_handle *h, const bs2e_config *configs,
                                         int64_t n_config, int64_t L, int64_t spin, int64_t full,
                                         int64_t *nnz_H, int64_t *nnz_S);
BS2E_API bs2e_status bs2e_block_fill_ex(bs2e_handle *h, const bs2e_config *configs,
                                        int64_t n_config, int64_t L, int64_t spin, int64_t full,
                                        int64_t *H_index_ptr, int64_t *H_indices, double *H_data,
                                        int64_t *S_index_ptr, int64_t *S_indices, double *S_data,
                                        int64_t out_on_device);

/* Every symmetry block of a basis in one call: replaces the OpenMP loop of
 * construct_block_tensor over bas%syms (main_basis_setup.f90:105-116), so a
 * shim can make one call outside any parallel region.  Block i is
 * (configs[i], n_config[i], L[i], spin[i]); full applies to all.
 * count_all writes nnz_H[i], nnz_S[i]; fill_all writes block i into
 * H_index_ptr[i], H_indices[i], H_data[i], S_index_ptr[i], S_indices[i],
 * S_data[i] (sized by the counts; host or device arrays as in
 * bs2e_block_fill_ex).  The blocks run one after another through the
 * single-block calls; counting first leaves up to 17 blocks (of at most 2^26
 * rows each) in the handle's block cache for the fills.  On failure the error
 * message starts with "block i:". */
BS2E_API bs2e_status bs2e_blocks_count_all(bs2e_handle *h, int64_t n_blocks,
                                           const bs2e_config *const *configs,
                                           const int64_t *n_config, const int64_t *L,
                                           const int64_t *spin, int64_t full, int64_t *nnz_H,
                                           int64_t *nnz_S);
BS2E_API bs2e_status bs2e_blocks_fill_all(bs2e_handle *h, int64_t n_blocks,
                                          const bs2e_config *const *configs,
                                          const int64_t *n_config, const int64_t *L,
                                          const int64_t *spin, int64_t full,
                                          int64_t *const *H_index_ptr, int64_t *const *H_indices,
                                          double *const *H_data, int64_t *const *S_index_ptr,
                                          int64_t *const *S_indices, double *const *S_data,
                                          int64_t out_on_device);

/* Configuration list of one symmetry block, as count_configs
 * (src/tools/orbital_tools.f90:119-216) with consistent() (:46-72); spin as
 * above.  Returns the count in *n_config and writes the list when out != NULL. */
BS2E_API bs2e_status bs2e_configs(int64_t L, int64_t parity_odd, int64_t max_l_1p, int64_t n_b,
                                  int64_t k, int64_t max_n_b, int64_t n_all_l, int64_t l2_max,
                                  int64_t spin, bs2e_config *out, int64_t *n_config);

/* ang_k_LS (src/tools/wigner_tools.f90:126-138) computed from exact rational
 * 3j/6j sums: confs(1) = (la, lb), confs(2) = (lc, ld). */
BS2E_API double bs2e_ang_k_LS(int64_t k, int64_t la, int64_t lb, int64_t lc, int64_t ld,
                              int64_t L);
/* Wigner 3j and 6j symbols of integer arguments (GSL's coupling functions as
 * used by wigner_tools.f90:30-60). */
BS2E_API double bs2e_three_j(int64_t ja, int64_t jb, int64_t jc, int64_t ma, int64_t mb,
                             int64_t mc);
BS2E_API double bs2e_six_j(int64_t ja, int64_t jb, int64_t jc, int64_t jd, int64_t je,
                           int64_t jf);

/* Radial dipole matrices on the device, as setup_radial_dip
 * (src/mat_els/mat_els.f90:120-170, 348-390): gauge 0 = length ('l', r_mat),
 * 1 = velocity ('v', dr_mat and r_inv_mat).  Needs bs2e_slater (tabulation).
 * Optional dense complex n_b x n_b copies out (NULL to skip). */
BS2E_API bs2e_status bs2e_radial_dipole(bs2e_handle *h, int64_t gauge, double *r_mat,
                                        double *dr_mat, double *r_inv_mat);

/* Uses caller-computed radial dipole matrices (type(radial_dipole) of
 * mat_els.f90:14-19): complex n_b x n_b column-major; length gauge needs r_mat,
 * velocity gauge dr_mat and r_inv_mat (the others may be NULL). */
BS2E_API bs2e_status bs2e_set_radial_dipole(bs2e_handle *h, int64_t gauge, const double *r_mat,
                                            const double *dr_mat, const double *r_inv_mat);

/* Dipole block between row symmetry (L1, M1, parity pi1) and column symmetry
 * (L2, M2, pi2) for polarisation q in {-1, 0, 1}: construct_dip_block_tensor
 * with init_dip_block (src/mat_els/dipole.f90:8-47, 87-146).  compute = 0
 * gives the empty block the reference stores for skipped pairs
 * (main_basis_setup.f90:133-137).  Uses the overlap S set by
 * bs2e_set_one_body / bs2e_one_body.  The fill writes a 1-based CSR of shape
 * n_rows x n_cols; an empty block gets index_ptr = 1 everywhere. */
BS2E_API bs2e_status bs2e_dip_block_count(bs2e_handle *h, const bs2e_config *rows, int64_t n_rows,
                                          int64_t L1, int64_t M1, int64_t pi1,
                                          const bs2e_config *cols, int64_t n_cols, int64_t L2,
                                          int64_t M2, int64_t pi2, int64_t q, int64_t compute,
                                          int64_t *nnz);
BS2E_API bs2e_status bs2e_dip_block_fill(bs2e_handle *h, const bs2e_config *rows, int64_t n_rows,
                                         int64_t L1, int64_t M1, int64_t pi1,
                                         const bs2e_config *cols, int64_t n_cols, int64_t L2,
                                         int64_t M2, int64_t pi2, int64_t q, int64_t compute,
                                         int64_t *index_ptr, int64_t *indices, double *data,
                                         int64_t out_on_device);

/* Writers of the reference's block CSR files in gfortran's unformatted
 * sequential format (4-byte record markers; records above 2147483639 bytes
 * split into subrecords with signed markers).
 * bs2e_write_block_diag writes a block_diag_CS as CS_block_diag_store does
 * (src/tools/block_tools.f90:458-485) -- H_diag.dat / S_diag.dat: n_blocks
 * diagonal blocks, shapes[2*i..2*i+1] = (rows, cols), nnz[i], and per block
 * the 1-based CSR arrays (index_ptr[i] rows+1, indices[i] nnz, data[i] nnz
 * complex128; ignored when nnz[i] = 0).
 * bs2e_write_block writes a block_CS as CS_block_store does (:386-415) --
 * D_q.dat: n_rows_b x n_cols_b blocks, block (i, j) at index i + n_rows_b*j.
 * max_subrecord <= 0 uses gfortran's default subrecord size. */
BS2E_API bs2e_status bs2e_write_block_diag(const char *path, int64_t n_blocks,
                                           const int64_t *shapes, const int64_t *nnz,
                                           const int64_t *const *index_ptr,
                                           const int64_t *const *indices,
                                           const double *const *data, int64_t max_subrecord);
BS2E_API bs2e_status bs2e_write_block(const char *path, int64_t n_rows_b, int64_t n_cols_b,
                                      const int64_t *shapes, const int64_t *nnz,
                                      const int64_t *const *index_ptr,
                                      const int64_t *const *indices, const double *const *data,
                                      int64_t max_subrecord);

/* Row ranges of a block, for blocks too large to hold at once: the same
 * configuration list, L, spin and full as bs2e_block_count_ex, and rows
 * [row_first, row_first + row_count).  count_rows returns the range's
 * non-zeros; fill_rows writes the range's CSR arrays with a range-local
 * 1-based index_ptr (row_count + 1 entries, index_ptr[0] = 1) and the block's
 * 1-based column indices, exactly the rows row_first.. of bs2e_block_fill_ex.
 * With host outputs (out_on_device = 0), here and in bs2e_block_fill[_ex],
 * the rows are assembled in chunks through two staging areas of at most
 * 8 GiB each in HBM, the device-to-host copy of one chunk overlapping the
 * assembly of the next.  No counterpart in the reference (its blocks are
 * built whole, hamiltonian.f90:106-283). */
BS2E_API bs2e_status bs2e_block_count_rows(bs2e_handle *h, const bs2e_config *configs,
                                           int64_t n_config, int64_t L, int64_t spin,
                                           int64_t full, int64_t row_first, int64_t row_count,
                                           int64_t *nnz_H, int64_t *nnz_S);
BS2E_API bs2e_status bs2e_block_fill_rows(bs2e_handle *h, const bs2e_config *configs,
                                          int64_t n_config, int64_t L, int64_t spin, int64_t full,
                                          int64_t row_first, int64_t row_count,
                                          int64_t *H_index_ptr, int64_t *H_indices,
                                          double *H_data, int64_t *S_index_ptr,
                                          int64_t *S_indices, double *S_data,
                                          int64_t out_on_device);

/* n1 bands of a block, for consumers that take a block piece by piece on the
 * device (config lists of 10^7 rows, terabytes of CSR): the band holds the
 * rows of EVERY channel whose n1 lies in [n1_first, n1_first + n1_count), in
 * block order (channel by channel).  Unlike a contiguous row range, whose rows
 * (n1, n2) each need their own R^k tile, a band gives every staged tile
 * (n_a, n_b) the rows of all channels that read it, as the whole-block fill
 * does.  band_count returns the band's row and non-zero counts and, when
 * per_n1 != NULL, per n1 of the range the triple (rows, nnz_H, nnz_S) in
 * per_n1[3*i .. 3*i+2] (for choosing bands that fit a buffer).  fill_band
 * writes the band's CSR (range-local 1-based index_ptr, n_rows + 1 entries;
 * the block's 1-based column indices) and, when rows != NULL (n_rows
 * entries), the 1-based block row of every band row.  out_on_device = 1: the
 * seven arrays are device arrays on the handle's device; 0: host arrays, the
 * band assembled in groups of whole channels (a band's rows are channel-major,
 * so a group is one slice of every output array) through the handle's two HBM
 * staging areas (bs2e_opts.stage_bytes), the copy of one group to the host
 * running beside the fill of the next; the band's slice of each channel must
 * fit one area (BS2E_ERR_ARG otherwise: choose a narrower band).  The same
 * configuration list, L, spin and full as bs2e_block_count_ex.  No
 * counterpart in the reference (its blocks are built whole,
 * hamiltonian.f90:106-283). */
BS2E_API bs2e_status bs2e_block_band_count(bs2e_handle *h, const bs2e_config *configs,
                                           int64_t n_config, int64_t L, int64_t spin,
                                           int64_t full, int64_t n1_first, int64_t n1_count,
                                           int64_t *n_rows, int64_t *nnz_H, int64_t *nnz_S,
                                           int64_t *per_n1);
BS2E_API bs2e_status bs2e_block_fill_band(bs2e_handle *h, const bs2e_config *configs,
                                          int64_t n_config, int64_t L, int64_t spin,
                                          int64_t full, int64_t n1_first, int64_t n1_count,
                                          int64_t *rows, int64_t *H_index_ptr,
                                          int64_t *H_indices, double *H_data,
                                          int64_t *S_index_ptr, int64_t *S_indices,
                                          double *S_data, int64_t out_on_device);

/* Host-side planning of band work (no device, no handle; safe to call from
 * any thread or rank).  Multi-GPU assembly hands each rank whole bands: the
 * blocks are independent and a band's rows are independent of every other
 * band's (no exchange step), so ranks fill disjoint bands and the rank that
 * needs whole blocks gathers them (bs2e_band_merge), as CS_from_block_diag
 * joins blocks (src/tools/block_tools.f90:289-348).
 *
 * bs2e_band_plan cuts every block into n1 bands whose CSR (24 bytes per
 * non-zero of H and S plus 16 bytes per row) fits max_bytes, from per-n1
 * counts (bs2e_block_band_count with per_n1): block b has n1 = 1..n1_max[b]
 * and per_n1[b] holds (rows, nnz_H, nnz_S) per n1.  Bands are then assigned
 * to n_ranks ranks, largest first to the least loaded rank (ties to the
 * lower rank), so every rank computes the same plan without communicating.
 * Band i is bands[5*i .. 5*i+4] = (block, n1_first, n1_count, owner rank,
 * bytes), blocks in order, n1 ascending; *n_bands is set even when cap is too
 * small (BS2E_ERR_ARG, nothing written).  A single n1 above max_bytes is an
 * error (BS2E_ERR_ARG). */
BS2E_API bs2e_status bs2e_band_plan(int64_t n_blocks, const int64_t *n1_max,
                                    const int64_t *const *per_n1, int64_t max_bytes,
                                    int64_t n_ranks, int64_t cap, int64_t *bands,
                                    int64_t *n_bands);
/* The 1-based block rows of band [n1_first, n1_first + n1_count) of a
 * configuration list in basis order (the rows bs2e_block_fill_band writes, in
 * the same order); rows may be NULL to count only. */
BS2E_API bs2e_status bs2e_band_rows(const bs2e_config *configs, int64_t n_config,
                                    int64_t n1_first, int64_t n1_count, int64_t *rows,
                                    int64_t *n_rows);
/* Joins bands of one block into the block's CSR (host arrays): band i has
 * n_rows[i] rows with 1-based block rows rows[i], range-local 1-based
 * index_ptr[i] (n_rows[i] + 1), indices[i] and complex128 data[i].  The
 * bands' rows must cover 1..n_config exactly once (BS2E_ERR_ARG otherwise);
 * out_index_ptr (n_config + 1), out_indices and out_data are sized by the
 * sum of the bands' non-zeros. */
BS2E_API bs2e_status bs2e_band_merge(int64_t n_config, int64_t n_bands, const int64_t *n_rows,
                                     const int64_t *const *rows,
                                     const int64_t *const *index_ptr,
                                     const int64_t *const *indices, const double *const *data,
                                     int64_t *out_index_ptr, int64_t *out_indices,
                                     double *out_data);

/* How many counted blocks the handle keeps besides the current one (0..16;
 * 16 at creation).  A kept block is reused when the same configuration list
 * is counted or filled again, skipping its planning and count pass; with 0
 * every block other than the last one counted is planned and counted anew,
 * as count_nnz runs once per block in basis_setup (hamiltonian.f90:348-416),
 * on the same device buffers.  Lowering the number frees the blocks beyond
 * it.  No counterpart in the reference. */
BS2E_API bs2e_status bs2e_set_block_cache(bs2e_handle *h, int64_t n_blocks);

/* Product of a 1-based CSR matrix (n_rows x n_cols, nnz entries, complex128
 * data) with a complex128 vector, as the solvers apply H and S:
 *   op 0: y = A x             CSR_mv     (src/tools/sparse_array_tools.f90:966-994)
 *   op 1: y = A^T x           CSR_T_mv   (:996-1031), no conjugation
 *   op 2: y = A x, A complex symmetric from its column >= row entries
 *                             CSR_mv_sym (:1033-1074, mkl_zcsrsymv 'U')
 * x has n_cols entries (n_rows for op 1), y n_rows (n_cols for op 1).
 * on_device = 1: every pointer is a CUDA device pointer on the handle's
 * device (e.g. blocks kept in HBM by bs2e_block_fill_ex); 0: host arrays,
 * staged through the handle's buffers.  Row pointers and column indices are
 * range-checked on the device (BS2E_ERR_ARG); the call returns when y is
 * complete.  Sums run in a different order from the reference's, so y agrees
 * with it to rounding (about 1e-16 of sum |a_ij x_j|). */
BS2E_API bs2e_status bs2e_csr_mv(bs2e_handle *h, int64_t op, int64_t n_rows, int64_t n_cols,
                                 int64_t nnz, const int64_t *index_ptr, const int64_t *indices,
                                 const double *data, const double *x, double *y,
                                 int64_t on_device);

/* One CSR matrix from an n_rb x n_cb block matrix of 1-based CSR blocks, as
 * CS_from_block / CSR_from_block do (src/tools/block_tools.f90:153-234): block
 * (i, j) (0-based) is entry b = i + n_rb*j of shapes (rows, cols pairs), nnz,
 * index_ptr, indices and data (complex128); blocks with nnz = 0 need no
 * arrays.  Row r of block row i is the concatenation over j of row r of
 * block (i, j), columns shifted by the widths of blocks (i, 0..j-1).  The
 * output has sum(rows of block (i, 0)) rows and sum(nnz) entries, sized by
 * the caller.  A block-diagonal matrix (CSR_from_block_diag, :289-348) is the
 * case with empty off-diagonal blocks of the right shapes.  on_device = 1:
 * the per-block pointers and the outputs are device pointers. */
BS2E_API bs2e_status bs2e_csr_from_blocks(bs2e_handle *h, int64_t n_rb, int64_t n_cb,
                                          const int64_t *shapes, const int64_t *nnz,
                                          const int64_t *const *index_ptr,
                                          const int64_t *const *indices,
                                          const double *const *data, int64_t *out_index_ptr,
                                          int64_t *out_indices, double *out_data,
                                          int64_t on_device);

/* Batched radial stage: bs2e_slater + bs2e_rk (every multipole) of n handles
 * -- bases of different order, spline count, knots, quadrature and multipole
 * range -- as four persistent kernels (tabulation, moments, pair totals, R^k
 * store) that each drain one work queue over all problems, largest R^k
 * store first.  The first bs2e_batch_run tunes the R^k kernel's threads per
 * CTA and queue grab size by timing each candidate (every candidate is a
 * complete pass) and captures the four stages in a CUDA graph; later runs
 * replay the graph.  After a run every handle is in the state bs2e_slater +
 * bs2e_rk(h, 0, max_k + 1) leaves it in, with bit-identical values.  The
 * handles must be distinct, on one device, and outlive the batch; the run
 * locks all of them.  No counterpart in the reference (one basis per
 * basis_setup run, mat_els.f90:172-292, sparse_array_tools.f90:452-493). */
typedef struct bs2e_batch bs2e_batch;
BS2E_API bs2e_status bs2e_batch_create(bs2e_handle *const *handles, int64_t n, bs2e_batch **out);
BS2E_API bs2e_status bs2e_batch_run(bs2e_batch *b);
/* The tuned R^k shape (threads per CTA; tiles per queue access, negative when
 * each CTA takes a fixed chunk instead of draining the queue), whether the
 * graph exists, and the kernels launched so far. */
BS2E_API bs2e_status bs2e_batch_tuning(const bs2e_batch *b, int64_t *rk_threads, int64_t *chunk,
                                       int64_t *graph_ready, int64_t *launches);
BS2E_API bs2e_status bs2e_batch_destroy(bs2e_batch *b);

/* The CUDA stream all work of the handle runs on (cudaStream_t as void*), the
 * number of kernels the handle has launched so far, and a full synchronize.
 * Device-pointer inputs (out_on_device / on_device calls) are read on this
 * stream without waiting for other streams: work that produces them on
 * another stream must be complete (or ordered before this stream with an
 * event) when the call is made.  Every entry point has finished its device
 * work on this stream when it returns. */
BS2E_API bs2e_status bs2e_stream(bs2e_handle *h, void **stream);

/* Recreates the handle's stream with a CUDA stream priority (a smaller number
 * is a higher priority; cudaDeviceGetStreamPriorityRange gives the range,
 * values outside it are refused with BS2E_ERR_ARG).  Waits for the handle's
 * work first; bs2e_stream returns the new stream afterwards.  For a handle
 * whose kernels should take SM slots ahead of another's, e.g. one that applies
 * bands while a second handle fills the next ones.  No counterpart in the
 * reference. */
BS2E_API bs2e_status bs2e_set_stream_priority(bs2e_handle *h, int64_t priority);
BS2E_API bs2e_status bs2e_launch_count(const bs2e_handle *h, int64_t *count);
BS2E_API bs2e_status bs2e_synchronize(bs2e_handle *h);

#ifdef __cplusplus
}
#endif
#endif /* BS2E_H */
