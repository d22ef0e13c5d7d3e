// bs2e_internal.h -- shared declarations of the GB300 two-electron library.
//
// Data layout in HBM (0-based indices; N = n_b basis splines, W = 2k-1,
// K1 = max_k+1, q = k_GL points per interval, n_iv breakpoint intervals):
//   tab_r   [n_iv][q]           outer quadrature radii of each interval
//   tab_B   [n_iv][q][k]        values of the k splines non-zero on the interval
//   tab_D2  [n_iv][q][k]        their second derivatives (one-body kinetic term)
//   tab_ri  [n_iv][q][q]        inner radii on [t_iv, r_P] for every outer point P
//   tab_Bi  [n_iv][q][q][k]     spline values at the inner radii
//   mom     [n_iv][K1][2][k][k] per-interval moments (0: int B B r^k, 1: int B B r^-(k+1))
//   dint    [n_iv][K1][k*k][k*k] same-interval 2-D integrals D(p=(i,i'), q=(j,j'))
//   dsym    [n_iv][K1][k*k][k*k] D(p, q) + D(q, p), the pair the R^k store adds
//   tot     [2][K1][N][W]       moments summed over all shared intervals of a pair
//   R       [N][N][tile]        R^k store, tile = [K1][W][W] padded to 16 bytes:
//                               R^k[a,b,c,d] at tile(a,b)[k][c-a+k-1][d-b+k-1]
// Band pairs (a,c) with |a-c|<k share the intervals [max(a,c)-k+2, min(a,c)+1]
// (clipped to [0,n_iv)); spline b0 is local index s = b0+1-iv on interval iv.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>
#include <vector>

#include "../../include/bs2e.h"

namespace bs2e {

constexpr int kMaxOrder = 16;  // B-spline order limit (the reference allows 20 in BVALUE_D)
constexpr int kMaxGL = 32;     // Gauss-Legendre points per interval
constexpr int kMaxK1 = 32;     // multipoles 0..31
// mixed R^k store: a slice maximum is scaled to [2^112, 2^113).  Weighted sums
// in the fill (angular weights below 2^3, at most 32 terms) stay below 2^120;
// values 2^214 below the maximum keep both FP32 words normal.
constexpr int kRkBias = 112;

// Per (row channel, column channel) coupling of one symmetry block.
struct PairInfo {
    int32_t flags;   // bit0 dir_ok, bit1 ex_ok, bit2 l_eq, bit3 l_eq_ex, bit4 sums gated per entry
    int32_t nd, nx;  // lengths of the direct / exchange multipole lists
    int32_t pad;
    double sgn;      // exchange sign (-1)^(l_c+l_d+L) (times -1 for the triplet)
};

constexpr int kMaxL = 64;    // l1, l2 < 64 (channel lookup table is kMaxL x kMaxL)
constexpr int kMaxCh = 256;  // channels per symmetry block
// counted blocks kept besides the current one (and their total rows)
constexpr int kBlockCache = 16;
constexpr int64_t kBlockCacheRows = (int64_t)1 << 26;

// Host-side plan of one symmetry block: its channels (in configuration
// order) and the angular coupling of every (row channel, column channel).
struct BlockPlan {
    int64_t n_config = 0, L = 0, spin = 0, full = 1;
    int n_ch = 0;
    std::vector<int> ch_l1, ch_l2, ch_start;  // channel angular momenta and first row
    std::vector<PairInfo> pairs;              // [n_ch][n_ch]
    std::vector<int8_t> pair_k;               // [n_ch][n_ch][2][K1]
    std::vector<double> pair_a;               // [n_ch][n_ch][2][K1]
    std::vector<float> pair_af;               // [n_ch][n_ch][2][K1][2] (hi, lo) for the mixed path
    bool gated = false;                       // some pair has PairInfo bit4 set
};

// Device side of the counted block.  The configuration list itself is the
// row table; segment tables give, per (channel c, n1), the first row and the
// n2 range, from which the rows of a tile (n_a, n_b) follow directly.
struct DevBlock {
    bs2e_config *cfg = nullptr, *cfg_new = nullptr;  // uploaded configurations (current, incoming)
    int64_t cfg_cap = 0, cfg_new_cap = 0;
    int4 *marks = nullptr;        // channel starts found on the device (row, l1, l2, -)
    int *lmap = nullptr;          // [kMaxL][kMaxL] -> channel index or -1
    int *chl = nullptr;           // [n_ch] l1 << 8 | l2
    int *seg = nullptr;           // base | lo | hi, each [n_ch][N+2]
    int64_t seg_cap = 0;
    PairInfo *pairs = nullptr;
    int8_t *pair_k = nullptr;
    double *pair_a = nullptr;
    float *pair_af = nullptr;
    int64_t pair_cap = 0;
    int64_t *cntH = nullptr, *cntS = nullptr;  // per-row counts
    int64_t cntH_cap = 0, cntS_cap = 0;
    int64_t *scan_tmp = nullptr;
    int64_t scan_cap = 0;
    unsigned long long *stats = nullptr;  // [0] error bits, [1..2] count_nnz H,S, [3..4] construct H,S, [5] marks
    int64_t nnzH = -1, nnzS = -1;
    // 1-based CSR pointers of the whole block (n + 1 each), built on demand
    // for band fills and kept with the block
    int64_t *pfxH = nullptr, *pfxS = nullptr;
    int64_t pfx_cap = 0;
    bool pfx_valid = false;
    // identity of the counted block
    bool valid = false;
    int64_t L = -1, spin = -1, full = -1, n = -1;
};

// Dipole coupling of one (row channel, column channel) pair: c[0..7] are the
// (alpha, beta) coefficients of the four one-particle terms, with the 3j
// factor, the 6j/sqrt factors and the exchange phase folded in.
struct DipPair {
    int32_t ok;
    int32_t tm;  // bit t: term t has a non-zero coefficient pair c[2t], c[2t+1]
    double c[8];
};

// Device view of one dipole block being assembled.
struct DipDev {
    const bs2e_config *rows = nullptr;
    int64_t n_rows = 0;
    const int *lmap_r = nullptr;
    int *seg = nullptr;  // column segment tables base | lo | hi
    int64_t nseg = 0;
    int n_ch_r = 0, n_ch_c = 0;
    const DipPair *pairs = nullptr;
    unsigned long long *stats = nullptr;
};

struct Radial {
    int k = 0, q = 0, K1 = 0, N = 0, n_iv = 0, W = 0, n = 0, n_knots = 0;
    int64_t tile = 0;  // padded doubles per R tile
};

}  // namespace bs2e

struct bs2e_handle {
    std::mutex mu;
    std::string err;
    int device = 0;
    int precision = 0;
    cudaStream_t stream = nullptr;
    int64_t launches = 0;
    bs2e::Radial g;
    std::vector<double> knots, glx, glw;
    // device radial data
    double *d_knots = nullptr, *d_glx = nullptr, *d_glw = nullptr;
    double *d_tab_D1 = nullptr;  // first derivatives (velocity-gauge dipoles)
    double *d_tab_r = nullptr, *d_tab_B = nullptr, *d_tab_D2 = nullptr, *d_tab_ri = nullptr,
           *d_tab_Bi = nullptr;
    double *d_mom = nullptr, *d_dint = nullptr, *d_dsym = nullptr, *d_tot = nullptr;
    double *d_R = nullptr;      // FP64 store
    float2 *d_Rf = nullptr;     // mixed store: scaled (hi, lo) pairs, same tile layout
    int32_t *d_Rexp = nullptr;  // mixed store: power-of-two scale per (tile, k)
    int *d_err = nullptr;       // device error word (bounded waits)
    bool slater_done = false;
    std::vector<char> rk_done;  // per k
    // one-body, banded complex: Hb[l][x][W], Sb[x][W]
    double2 *d_Hb = nullptr, *d_Sb = nullptr;
    float4 *d_Hbf = nullptr, *d_Sbf = nullptr;  // same bands as FP32 pairs (mixed path)
    unsigned long long *d_range = nullptr;      // min / max magnitude of the H and S bands
    int64_t n_l = 0;
    bool have_one_body = false;
    bool s_real = true;
    bool ff_one_body = false;  // mixed path may use the FP32-pair bands
    // the block counted last (plan + device state) and up to kBlockCache
    // earlier ones, most recently used first
    bs2e::BlockPlan plan;
    bs2e::DevBlock blk;
    std::vector<std::pair<bs2e::DevBlock, bs2e::BlockPlan>> parked;
    int cache_max = bs2e::kBlockCache;  // parked blocks kept (bs2e_set_block_cache)
    // band fills: per channel (first row, local row offset) and gather scratch
    int *d_band = nullptr;
    int64_t *d_band_idx = nullptr, *d_band_val = nullptr;
    int64_t band_cap = 0;
    int64_t *d_bptr = nullptr;  // band pointers (H, S, rows) of host-output band fills
    int64_t bptr_cap = 0;
    // radial dipole bands (M1, M2) and dipole-block work buffers
    double2 *d_dM1 = nullptr, *d_dM2 = nullptr;
    int dip_gauge = -1;
    int dip_kind = 0;  // radial dipole bands: 1 all real, 2 all imaginary, 0 general
    bs2e_config *d_dip_rows = nullptr, *d_dip_cols = nullptr;
    int64_t dip_rows_cap = 0, dip_cols_cap = 0;
    int *d_dip_lmap = nullptr, *d_dip_seg = nullptr;
    int64_t dip_seg_cap = 0;
    bs2e::DipPair *d_dip_pairs = nullptr;
    int64_t dip_pairs_cap = 0;
    int4 *d_dip_marks = nullptr;
    unsigned long long *d_dip_stats = nullptr;
    int64_t *d_dip_cnt = nullptr, *d_dip_part = nullptr;
    int64_t dip_cnt_cap = 0, dip_part_cap = 0;
    // host-output fills: range CSR pointers, two staging areas in HBM and the
    // stream that copies a filled area to the host while the next one fills
    int64_t *d_rptrH = nullptr, *d_rptrS = nullptr;
    int64_t rptr_cap = 0;
    unsigned char *d_stage[2] = {nullptr, nullptr};
    int64_t stage_cap = 0;
    int64_t stage_limit = (int64_t)8 << 30;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_filled[2] = {nullptr, nullptr}, ev_copied[2] = {nullptr, nullptr};
    // mat-vec staging for host operands, and its bad-input flag word
    int64_t *d_mv_ptr = nullptr, *d_mv_idx = nullptr;
    double2 *d_mv_A = nullptr, *d_mv_x = nullptr, *d_mv_y = nullptr;
    int64_t mv_ptr_cap = 0, mv_idx_cap = 0, mv_A_cap = 0, mv_x_cap = 0, mv_y_cap = 0;
    int *d_mv_bad = nullptr;
};

namespace bs2e {

// Host helpers (bs2e_angular.cpp, bs2e_basis.cpp)
double ang_k_LS(int k, int la, int lb, int lc, int ld, int L);
double three_j(int ja, int jb, int jc, int ma, int mb, int mc);
double six_j(int ja, int jb, int jc, int jd, int je, int jf);
void gauss_legendre(int q, double *x, double *w);
// Angular tables of a block from its ordered channel list.
void plan_channels(BlockPlan &plan, int K1);

// Scratch of the allocation-free R^k lookup (bs2e_noalloc.cu): resolves its
// device address on `device` and loads its kernel (bs2e_create calls this).
cudaError_t noalloc_prepare(int device, bool refresh);

// Kernel launchers (bs2e_radial.cu)
// Device view of one handle's radial buffers (the single-handle kernels and
// the batched ones read the same struct).
struct RadialDev {
    const double *knots, *glx, *glw;
    double *tab_r, *tab_B, *tab_D2, *tab_D1, *tab_ri, *tab_Bi;
    double *mom, *dint, *dsym, *tot, *R;
    float2 *Rf;
    int *Rexp;
    int k, q, K1, N, n_iv, mixed;
    int64_t tile;
};
RadialDev radial_dev(const bs2e_handle *h);
// batched radial stages (0 tabulate, 1 moments, 2 totals, 3 R^k store)
int radial_batch_blocks_per_sm(int stage, int threads, size_t smem);
void launch_radial_batch(cudaStream_t s, int stage, int grid, int threads, size_t smem,
                         const RadialDev *probs, const int64_t *off, int n,
                         unsigned long long *counter, int chunk, int persistent);
size_t moments_smem(const Radial &g);
size_t rk_store_smem(const Radial &g, bool mixed);
void launch_tabulate(bs2e_handle *h);
void launch_moments(bs2e_handle *h);
void launch_totals(bs2e_handle *h);
void launch_rk_fill(bs2e_handle *h, int k_first, int k_count);
void launch_rk_gather(bs2e_handle *h, int64_t n, const int64_t *d_keys, double *d_vals);
void launch_rk_slice(bs2e_handle *h, int kk, double *d_out);
void launch_one_body(bs2e_handle *h, int64_t Z, int64_t n_l, int64_t cap_order, double cap_r0,
                     double eta_re, double eta_im);
void launch_band_split(bs2e_handle *h);
// One block of a block matrix being joined into one CSR (device pointers).
struct CatBlock {
    const int64_t *ptr, *idx;
    const double2 *data;
    int64_t nnz, n_cols, col0;
};
struct CatArgs {
    const CatBlock *blocks;  // [n_rb * n_cb], block (i, j) at i + n_rb * j
    const int64_t *row0;     // [n_rb + 1] first output row of each block row
    int n_rb, n_cb;
    int64_t n_rows;
};
// copy = false: row lengths into cnt and the 1-based index_ptr into optr;
// copy = true: the entries into oidx / odat
void launch_cat(bs2e_handle *h, const CatArgs &A, int64_t *cnt, int64_t *part, int64_t *optr,
                int64_t *oidx, double2 *odat, int *bad, bool copy);
void scan_one(bs2e_handle *h, const int64_t *in, int64_t n, int64_t *part, int64_t *ptr);
void launch_csr_mv(bs2e_handle *h, int op, int64_t n_rows, int64_t n_cols, int64_t nnz,
                   const int64_t *ptr, const int64_t *idx, const double2 *A, const double2 *x,
                   double2 *y, int *bad);
// Kernel launchers (bs2e_dipole.cu)
void launch_radial_dip(bs2e_handle *h, int gauge);
void launch_dip_count(bs2e_handle *h, const DipDev &D, int64_t *cnt);
void launch_dip_fill(bs2e_handle *h, const DipDev &D, const int64_t *ptr, int64_t *idx,
                     double2 *dat);
// Kernel launchers (bs2e_assembly.cu)
void launch_cfg_equal(bs2e_handle *h, const bs2e_config *a, const bs2e_config *b, int64_t n,
                      unsigned long long *stats);
void launch_chan_marks(bs2e_handle *h, int64_t n);
void launch_plan_seg(bs2e_handle *h, int64_t n);
void launch_block_count(bs2e_handle *h);
void launch_chan_marks_on(bs2e_handle *h, const bs2e_config *cfg, int64_t n, int4 *marks, int cap,
                          unsigned long long *stats);
void launch_plan_seg_on(bs2e_handle *h, const bs2e_config *cfg, int64_t n, const int *lmap,
                        int segS, int *base, int *lo, int *hi, unsigned long long *stats);
void scan_one(bs2e_handle *h, const int64_t *in, int64_t n, int64_t *part, int64_t *ptr);
// Rows [row0, row1) of the counted block; their tiles have n_a in [a0, a1].
// Row r's entries start at output position ptr[r - ptr_row0] - 1 - base.
// rows_mode: a warp per row with the R^k tile read through L1/L2 (ranges
// inside one or two channels, where each tile holds a single row of the
// range) instead of a CTA per staged tile.
// band (device, 2 x n_ch ints, or null): a band fill, where row r of channel
// c is local row band[n_ch + c] + (r - band[c]) of the output, whose pointers
// start at ptr[0] = 1.
struct FillRange {
    int64_t row0 = 0, row1 = 0, ptr_row0 = 0, Hbase = 0, Sbase = 0;
    int a0 = 1, a1 = 0;
    bool rows_mode = false;
    const int *band = nullptr;
    int64_t band_rows = 0;  // rows of the band when band is set
    int ch0 = 0, ch1 = -1;  // only rows of channels [ch0, ch1) (ch1 < 0: all)
};
// out[i] = src[idx[i]] for i < n (device arrays)
void launch_gather_i64(bs2e_handle *h, const int64_t *src, const int64_t *idx, int64_t n,
                       int64_t *out);
// Band-local 1-based pointers of a band of n_rows rows: band (device, 2 x n_ch
// ints as in FillRange) and boff (device, 2 x n_ch int64: H and S non-zeros of
// the band before channel c); rows (may be null) gets the 1-based block rows.
void launch_band_ptr(bs2e_handle *h, const int *band, const int64_t *boff, int n_ch,
                     int64_t n_rows, int64_t *Hptr, int64_t *Sptr, int64_t *rows);
// 1-based CSR pointers of rows [row0, row0 + n) (n + 1 entries, starting at 1)
void launch_block_scan(bs2e_handle *h, int64_t *d_Hptr, int64_t *d_Sptr, int64_t row0,
                       int64_t n);
void launch_block_fill(bs2e_handle *h, const FillRange &r, const int64_t *d_Hptr,
                       const int64_t *d_Sptr, int64_t *d_Hidx, double2 *d_Hdat, int64_t *d_Sidx,
                       double2 *d_Sdat);

}  // namespace bs2e
