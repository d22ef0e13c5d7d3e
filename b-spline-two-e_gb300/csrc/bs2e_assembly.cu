// bs2e_assembly.cu -- CSR assembly of one symmetry block of H and S.
//
// Reference: construct_block_tensor and count_nnz
// (src/mat_els/hamiltonian.f90:106-283, 348-416), c_mat_neq_tens / r_12_tens
// (src/mat_els/mat_els.f90:552-571, 608-633), H_1p_neq and S_mat_neq
// (mat_els.f90:664-678, 697-715).
//
// For row i = (channel c_r; n_a, n_b) and column j = (channel c_c; n_c, n_d):
//   sup  = |n_a-n_c|<k and |n_b-n_d|<k        sup_x = |n_a-n_d|<k and |n_b-n_c|<k
//   r12  = (sup and dir_ok) or (sup_x and ex_ok)  (dir_ok / ex_ok: some |ang_k| > 5e-15)
//   H(i,j) stored   iff (sup or sup_x) and (r12 or l_eq or l_eq_ex)
//   S(i,j) stored   iff (sup and l_eq) or (sup_x and l_eq_ex)
// so in column channel c_c the columns of a row are (n_c, n_d) in
// (A x B) u (B x A), A = [n_a-k+1, n_a+k-1], B = [n_b-k+1, n_b+k-1], clipped to
// the configurations of c_c -- at most two n_d intervals per n_c.  Columns come
// out ascending because configurations are ordered channel, n1, n2.
//
// The fill kernel runs one CTA per (n_a, n_b) tile: the R^k tile
// R[n_a][n_b][k][*][*] is staged into shared memory by one bulk TMA copy and
// serves every row with that (n_a, n_b) -- the direct term reads
// R[k][n_c-n_a+k-1][n_d-n_b+k-1], the exchange term R[k][n_d-n_a+k-1][n_c-n_b+k-1].
// One warp assembles one row; lanes enumerate the (n_c, n_d) runs of a column
// channel, a warp scan gives run offsets and each lane finds its run by a
// 5-step shuffle search, so stores of a row are contiguous and coalesced.
#include <cuda_runtime.h>

#include "bs2e_internal.h"
#include "bs2e_device.cuh"

namespace bs2e {
namespace {

struct BlockArgs {
    const bs2e_config *cfg;                 // the configuration list (row table)
    const int *lmap;                        // [kMaxL][kMaxL] channel of (l1, l2)
    const int *chl;                         // [n_ch] l1 << 8 | l2
    const int *seg_base, *seg_lo, *seg_hi;  // [n_ch][N+2]
    const PairInfo *pairs;
    const int8_t *pair_k;
    const double *pair_a;
    const float *pair_af;  // (hi, lo) FP32 pairs of pair_a
    int n_ch, N, k, K1, full, segS;
    int64_t n_rows;
};

// Column set of row (n_a, n_b) in channel c_c for n_c: H set and S set.
__device__ __forceinline__ void col_sets(const BlockArgs &A, int c_r, int c_c, int n_a, int n_b,
                                         int n_c, int flags, Iv2 &hset, Iv2 &sset, int &base,
                                         int &lo) {
    const int k = A.k;
    size_t s = (size_t)c_c * A.segS + n_c;
    base = A.seg_base[s];
    lo = A.seg_lo[s];
    int hi = A.seg_hi[s];
    int lo2 = lo;
    if (!A.full && c_c == c_r && n_c == n_a) lo2 = max(lo2, n_b);  // upper triangle: j >= i
    bool dir_ok = flags & 1, ex_ok = flags & 2, leq = flags & 4, leqx = flags & 8;
    bool Aok = dir_ok || leq || leqx, Bok = ex_ok || leq || leqx;
    bool in_a = abs(n_c - n_a) < k, in_b = abs(n_c - n_b) < k;
    int x10 = max(n_b - k + 1, lo2), x11 = min(n_b + k - 1, hi);
    int x20 = max(n_a - k + 1, lo2), x21 = min(n_a + k - 1, hi);
    if (hi < lo2 || base < 0) {
        hset = Iv2{0, 0, 0, 0};
        sset = hset;
        return;
    }
    hset = make_union(x10, x11, Aok && in_a, x20, x21, Bok && in_b);
    sset = make_union(x10, x11, leq && in_a, x20, x21, leqx && in_b);
}

// ---------------------------------------------------------------------------
// Count.  cnt_H / cnt_S use the construct predicate; the totals of the
// count_nnz predicate (hamiltonian.f90:386-413) are accumulated in stats[1..2]
// (construct totals in stats[3..4]) so the host can detect a block where the
// two disagree.
// ---------------------------------------------------------------------------

// Counts of row (c_r, n_a, n_b) in column channel c_c: construct H and S
// entries and the count_nnz H and S entries.
__device__ __forceinline__ void count_pair(const BlockArgs &A, int c_r, int c_c, int n_a, int n_b,
                                           int64_t &ch, int64_t &cs, long long &refH,
                                           long long &refS) {
    const int k = A.k;
    const int flags = A.pairs[(size_t)c_r * A.n_ch + c_c].flags;
    const bool dir_ok = flags & 1, ex_ok = flags & 2, leq = flags & 4, leqx = flags & 8;
    const int nlo = (!A.full && c_c == c_r) ? n_a : 1;
    const Iv2 cand = nc_candidates(n_a, n_b, k, A.N, true, true, nlo);
    const int ncand = cand.l1 + cand.l2;
    for (int t = 0; t < ncand; ++t) {
        const int n_c = iv2_at(cand, t);
        Iv2 hs, ss;
        int base, lo;
        col_sets(A, c_r, c_c, n_a, n_b, n_c, flags, hs, ss, base, lo);
        ch += hs.l1 + hs.l2;
        cs += ss.l1 + ss.l2;
        // count_nnz semantics: sup entries count if dir_ok, sup_x-only entries if ex_ok
        const size_t s = (size_t)c_c * A.segS + n_c;
        int lo2 = A.seg_lo[s];
        const int hi = A.seg_hi[s];
        if (A.seg_base[s] < 0) continue;
        if (!A.full && c_c == c_r && n_c == n_a) lo2 = max(lo2, n_b);
        if (hi < lo2) continue;
        const bool in_a = abs(n_c - n_a) < k, in_b = abs(n_c - n_b) < k;
        const int ysup = in_a ? ovl(n_b - k + 1, n_b + k - 1, lo2, hi) : 0;
        const int yx = in_b ? ovl(n_a - k + 1, n_a + k - 1, lo2, hi) : 0;
        const int both = (in_a && in_b) ? max(0, min(min(n_b + k - 1, n_a + k - 1), hi) -
                                                     max(max(n_b - k + 1, n_a - k + 1), lo2) + 1)
                                        : 0;
        const int xonly = yx - both;
        refH += (dir_ok ? ysup : 0) + (ex_ok ? xonly : 0);
        refS += (leq ? ysup : 0) + (leqx ? xonly : 0);
    }
}

// One CTA per (n_a, n_b) tile, all rows of the tile at once.  Over column
// channel c_c a row's sets depend on its own channel only through the pair
// flags: the H set is A (the direct window [n_b - k + 1, n_b + k - 1], where
// |n_c - n_a| < k) if Aok, B (the exchange window around n_a, where
// |n_c - n_b| < k) if Bok, their union if both; the S set likewise with leq
// and leqx; the count_nnz H count is dir_ok |A| + ex_ok |B \ A| and the S
// count leq |A| + leqx |B \ A|.  So the tile sums SA = sum |A|, SB = sum |B|
// and SAB = sum |A u B| over the candidates n_c, once per column channel,
// give every row's counts (|B \ A| sums to SAB - SA) -- exactly the numbers
// the per-row loop of count_pair adds up, at a few percent of its work (the
// tile's 20-60 rows share the sums).  Without `full`, a row's own channel
// takes only n_c >= n_a and its upper triangle, so that pair runs
// count_pair.
__global__ void __launch_bounds__(128) k_csr_count_tiles(BlockArgs A, int a0,
                                                         int64_t *__restrict__ cntH,
                                                         int64_t *__restrict__ cntS,
                                                         unsigned long long *__restrict__ stats) {
    __shared__ int sSA[kMaxCh], sSB[kMaxCh], sSAB[kMaxCh];
    __shared__ int srow[kMaxCh], sch[kMaxCh], snrow;
    const int k = A.k;
    const int n_a = a0 + (int)(blockIdx.x / A.N), n_b = blockIdx.x % A.N + 1;
    if (threadIdx.x == 0) snrow = 0;
    __syncthreads();
    for (int c = threadIdx.x; c < A.n_ch; c += blockDim.x) {
        const size_t s = (size_t)c * A.segS + n_a;
        const int base = A.seg_base[s], lo = A.seg_lo[s], hi = A.seg_hi[s];
        if (base >= 0 && lo <= n_b && n_b <= hi) {
            const int slot = atomicAdd(&snrow, 1);
            srow[slot] = base + (n_b - lo);
            sch[slot] = c;
        }
    }
    __syncthreads();
    const int nrow = snrow;
    if (nrow == 0) return;
    const Iv2 cand = nc_candidates(n_a, n_b, k, A.N, true, true, 1);
    const int ncand = cand.l1 + cand.l2;
    for (int c_c = threadIdx.x; c_c < A.n_ch; c_c += blockDim.x) {
        int sa = 0, sb = 0, sab = 0;
        for (int t = 0; t < ncand; ++t) {
            const int n_c = iv2_at(cand, t);
            const size_t s = (size_t)c_c * A.segS + n_c;
            const int base = A.seg_base[s], lo = A.seg_lo[s], hi = A.seg_hi[s];
            if (base < 0 || hi < lo) continue;
            const bool in_a = abs(n_c - n_a) < k, in_b = abs(n_c - n_b) < k;
            const int x10 = max(n_b - k + 1, lo), x11 = min(n_b + k - 1, hi);
            const int x20 = max(n_a - k + 1, lo), x21 = min(n_a + k - 1, hi);
            const Iv2 u = make_union(x10, x11, in_a, x20, x21, in_b);
            sa += in_a ? max(0, x11 - x10 + 1) : 0;
            sb += in_b ? max(0, x21 - x20 + 1) : 0;
            sab += u.l1 + u.l2;
        }
        sSA[c_c] = sa;
        sSB[c_c] = sb;
        sSAB[c_c] = sab;
    }
    __syncthreads();
    long long refH = 0, refS = 0, totH = 0, totS = 0;
    for (int r = threadIdx.x; r < nrow; r += blockDim.x) {
        const int c_r = sch[r];
        int64_t ch = 0, cs = 0;
        const PairInfo *pr = A.pairs + (size_t)c_r * A.n_ch;
        for (int c_c = A.full ? 0 : c_r + 1; c_c < A.n_ch; ++c_c) {
            const int flags = pr[c_c].flags;
            const bool dir_ok = flags & 1, ex_ok = flags & 2, leq = flags & 4, leqx = flags & 8;
            const bool Aok = dir_ok || leq || leqx, Bok = ex_ok || leq || leqx;
            const int sa = sSA[c_c], sb = sSB[c_c], sab = sSAB[c_c];
            ch += Aok ? (Bok ? sab : sa) : (Bok ? sb : 0);
            cs += leq ? (leqx ? sab : sa) : (leqx ? sb : 0);
            refH += (dir_ok ? sa : 0) + (ex_ok ? sab - sa : 0);
            refS += (leq ? sa : 0) + (leqx ? sab - sa : 0);
        }
        if (!A.full) count_pair(A, c_r, c_r, n_a, n_b, ch, cs, refH, refS);
        cntH[srow[r]] = ch;
        cntS[srow[r]] = cs;
        totH += ch;
        totS += cs;
    }
    for (int o = 16; o > 0; o >>= 1) {
        refH += __shfl_down_sync(0xffffffffu, refH, o);
        refS += __shfl_down_sync(0xffffffffu, refS, o);
        totH += __shfl_down_sync(0xffffffffu, totH, o);
        totS += __shfl_down_sync(0xffffffffu, totS, o);
    }
    if ((threadIdx.x & 31) == 0 && (refH || refS || totH || totS)) {
        atomicAdd(&stats[1], (unsigned long long)refH);
        atomicAdd(&stats[2], (unsigned long long)refS);
        atomicAdd(&stats[3], (unsigned long long)totH);
        atomicAdd(&stats[4], (unsigned long long)totS);
    }
}

// ---------------------------------------------------------------------------
// Device-side planning of a block from its configuration list.
// stats[0] error bits: 1 = n or l out of range, 2 = not in basis order.
// ---------------------------------------------------------------------------
__global__ void k_cfg_equal(const bs2e_config *__restrict__ a, const bs2e_config *__restrict__ b,
                            int64_t n, unsigned long long *__restrict__ stats) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const bs2e_config x = a[i], y = b[i];
        if (x.n1 != y.n1 || x.n2 != y.n2 || x.l1 != y.l1 || x.l2 != y.l2 || x.eqv != y.eqv)
            atomicOr(&stats[6], 1ull);
    }
}

// Rows where a new channel (l1, l2) starts, appended in any order.
__global__ void k_chan_marks(const bs2e_config *__restrict__ cfg, int64_t n, int N,
                             int4 *__restrict__ marks, int cap,
                             unsigned long long *__restrict__ stats) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const bs2e_config c = cfg[i];
        if (c.n1 < 1 || c.n1 > N || c.n2 < 1 || c.n2 > N || c.l1 < 0 || c.l2 < 0 ||
            c.l1 >= kMaxL || c.l2 >= kMaxL) {
            atomicOr(&stats[0], 1ull);
            continue;
        }
        bool start = (i == 0) || cfg[i - 1].l1 != c.l1 || cfg[i - 1].l2 != c.l2;
        if (start) {
            unsigned long long slot = atomicAdd(&stats[5], 1ull);
            if (slot < (unsigned long long)cap) marks[slot] = make_int4((int)i, (int)c.l1, (int)c.l2, 0);
        }
    }
}

// Segment tables and basis-order checks: within a channel n1 ascends, and the
// n2 of one (channel, n1) group are consecutive.
__global__ void k_plan_seg(const bs2e_config *__restrict__ cfg, int64_t n, const int *__restrict__ lmap,
                           int segS, int *__restrict__ seg_base, int *__restrict__ seg_lo,
                           int *__restrict__ seg_hi, unsigned long long *__restrict__ stats) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const bs2e_config c = cfg[i];
        if (c.l1 < 0 || c.l2 < 0 || c.l1 >= kMaxL || c.l2 >= kMaxL) continue;  // flagged already
        const int ch = lmap[c.l1 * kMaxL + c.l2];
        bool new_ch = (i == 0) || cfg[i - 1].l1 != c.l1 || cfg[i - 1].l2 != c.l2;
        bool new_grp = new_ch || cfg[i - 1].n1 != c.n1;
        if (!new_ch) {
            const bs2e_config p = cfg[i - 1];
            if (new_grp ? !(c.n1 > p.n1) : (c.n2 != p.n2 + 1)) atomicOr(&stats[0], 2ull);
        }
        bool last = (i == n - 1) || cfg[i + 1].l1 != c.l1 || cfg[i + 1].l2 != c.l2 ||
                    cfg[i + 1].n1 != c.n1;
        size_t s = (size_t)ch * segS + (size_t)c.n1;
        if (new_grp) {
            seg_base[s] = (int)i;
            seg_lo[s] = (int)c.n2;
        }
        if (last) seg_hi[s] = (int)c.n2;
    }
}

// ---------------------------------------------------------------------------
// Exclusive scan of int64 counts -> 1-based CSR pointers (three passes).
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 1024, kScanItems = 4, kScanTile = kScanThreads * kScanItems;

__device__ int64_t block_excl_scan(int64_t v, int64_t *ws, int64_t &total) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int64_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int64_t s = (lane < (int)(blockDim.x >> 5)) ? ws[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        ws[lane] = s;
    }
    __syncthreads();
    int64_t pre = (wid > 0) ? ws[wid - 1] : 0;
    total = ws[(blockDim.x >> 5) - 1];
    __syncthreads();
    return pre + x - v;
}

__global__ void k_scan_partials(const int64_t *__restrict__ in, int64_t n,
                                int64_t *__restrict__ part) {
    __shared__ int64_t ws[32];
    int64_t base = (int64_t)blockIdx.x * kScanTile;
    int64_t s = 0;
    for (int i = 0; i < kScanItems; ++i) {
        int64_t idx = base + (int64_t)threadIdx.x * kScanItems + i;
        if (idx < n) s += in[idx];
    }
    int64_t total;
    block_excl_scan(s, ws, total);
    if (threadIdx.x == 0) part[blockIdx.x] = total;
}

__global__ void k_scan_part_prefix(int64_t *__restrict__ part, int64_t nparts) {
    __shared__ int64_t ws[32];
    int64_t carry = 0;
    for (int64_t base = 0; base < nparts; base += blockDim.x) {
        int64_t idx = base + threadIdx.x;
        int64_t v = idx < nparts ? part[idx] : 0;
        int64_t total;
        int64_t ex = block_excl_scan(v, ws, total);
        if (idx < nparts) part[idx] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) part[nparts] = carry;
}

__global__ void k_scan_final(const int64_t *__restrict__ in, int64_t n,
                             const int64_t *__restrict__ part, int64_t *__restrict__ ptr) {
    __shared__ int64_t ws[32];
    int64_t base = (int64_t)blockIdx.x * kScanTile;
    int64_t v[kScanItems];
    int64_t s = 0;
    for (int i = 0; i < kScanItems; ++i) {
        int64_t idx = base + (int64_t)threadIdx.x * kScanItems + i;
        v[i] = idx < n ? in[idx] : 0;
        s += v[i];
    }
    int64_t total;
    int64_t ex = block_excl_scan(s, ws, total) + part[blockIdx.x];
    for (int i = 0; i < kScanItems; ++i) {
        int64_t idx = base + (int64_t)threadIdx.x * kScanItems + i;
        if (idx < n) ptr[idx] = ex + 1;  // 1-based
        ex += v[i];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) ptr[n] = part[gridDim.x] + 1;
}

// ---------------------------------------------------------------------------
// Fill.
// ---------------------------------------------------------------------------
struct FillArgs {
    BlockArgs B;
    const double *R;
    const float2 *Rf;  // mixed store (scaled FP32 pairs) and its per-(tile, k) exponents
    const int *Rexp;
    int64_t tile;
    const double2 *Hb, *Sb;
    const float4 *Hbf, *Sbf;  // the same bands as FP32 pairs (re hi, re lo, im hi, im lo)
    int s_real;
    int gated;                // 1: some channel pair needs the per-entry r_12_allowed test
    int ff_one_body;          // 1: mixed path may use Hbf/Sbf (S real, magnitudes in range)
    // rows [row0, row1) are filled; row r starts at output position
    // Hptr[x] - 1 - Hbase (likewise S), 1-based CSR pointers, where x is
    // r - ptr_row0, or in a band fill band[n_ch + c] + (r - band[c]) for r in
    // channel c
    const int64_t *Hptr, *Sptr;
    int64_t row0, row1, ptr_row0, Hbase, Sbase;
    const int *band;
    int64_t band_rows;  // rows of the band (pointer slots 0..band_rows)
    int ch0, ch1;       // only rows of channels [ch0, ch1) are filled
    int a0;  // tile (n_a, n_b) of CTA x: n_a = a0 + x / N, n_b = x % N + 1
    int64_t *Hidx, *Sidx;
    double2 *Hdat, *Sdat;
    int *err;
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) {
    return make_double2(a.x + b.x, a.y + b.y);
}
// banded one-body lookup M[x][y] (1-based), zero outside the band
__device__ __forceinline__ double2 band(const double2 *M, int N, int k, int x, int y) {
    int d = y - x;
    if (abs(d) >= k) return make_double2(0.0, 0.0);
    return M[(size_t)(x - 1) * (2 * k - 1) + (d + k - 1)];
}

__device__ __forceinline__ float4 bandf(const float4 *M, int k, int x, int y) {
    int d = y - x;
    if (abs(d) >= k) return make_float4(0.f, 0.f, 0.f, 0.f);
    return M[(size_t)(x - 1) * (2 * k - 1) + (d + k - 1)];
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Stages the R^k tile of (a, b) into shared memory with one bulk TMA copy.
// The wait is bounded (~4e9 cycles); on expiry the error word is set and the
// CTA waits a second bounded period for the copy before giving up.
__device__ bool stage_tile(const double *src, double *dst, uint32_t bytes, uint64_t *bar,
                           int *err) {
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                     "r"(bytes)
                     : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
            "[%3];" ::"r"(smem_u32(dst)),
            "l"(src), "r"(bytes), "r"(smem_u32(bar))
            : "memory");
    }
    long long t0 = clock64();
    bool done = false;
    while (!(done = mbar_try_wait(bar, 0))) {
        if (clock64() - t0 > 4000000000LL) break;
    }
    if (!done) {
        atomicExch(err, 1);
        long long t1 = clock64();
        while (!mbar_try_wait(bar, 0)) {
            if (clock64() - t1 > 4000000000LL) break;
        }
        return false;
    }
    return true;
}

// ---- FP32-pair (double-float) arithmetic of the mixed path ----------------
struct FF {
    float s, c;
};

// acc += a * x for double-float a, x; the product error is captured exactly
// with fmaf and the sum by TwoSum, so the pair keeps ~44 bits.
__device__ __forceinline__ void ff_madd(FF &acc, float2 a, float2 x) {
    float p = __fmul_rn(a.x, x.x);
    float e = fmaf(a.x, x.x, -p);
    e = fmaf(a.x, x.y, e);
    e = fmaf(a.y, x.x, e);
    float t = __fadd_rn(acc.s, p);
    float bp = __fsub_rn(t, acc.s);
    float err = __fadd_rn(__fsub_rn(acc.s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
    acc.s = t;
    acc.c = __fadd_rn(acc.c, __fadd_rn(err, e));
}

// x with its sign bit flipped when bit is the sign bit: multiplication by an
// exchange sign of +-1 as one integer operation instead of an FP64 one.
__device__ __forceinline__ double flip_sign(double x, long long bit) {
    return __longlong_as_double(__double_as_longlong(x) ^ bit);
}

// 2^n as float for -126 <= n <= 127, 0 below.
__device__ __forceinline__ float pow2f(int n) {
    return n < -126 ? 0.0f : __int_as_float((127 + min(n, 127)) << 23);
}

__device__ __forceinline__ FF two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float bp = __fsub_rn(s, a);
    float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
    return FF{s, e};
}

// Exact product a*b of two FP32 pairs up to the lo*lo term, unnormalised.
__device__ __forceinline__ FF ff_mul(float2 a, float2 b) {
    float p = __fmul_rn(a.x, b.x);
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    return FF{p, e};
}

__device__ __forceinline__ FF ff_add(FF a, FF b) {
    FF t = two_sum(a.s, b.s);
    t.c = __fadd_rn(t.c, __fadd_rn(a.c, b.c));
    return t;
}

__device__ __forceinline__ FF ff_neg_if(FF a, bool neg) {
    return neg ? FF{-a.s, -a.c} : a;
}

// (s + c) * 2^shift as a double, assembled from the bit patterns with integer
// instructions only (no FP64 operation): after TwoSum |c| <= ulp(s)/2, so the
// leading part is s with its exponent rebased and its significand widened,
// and c enters as an integer multiple of the double's ulp (its bits below that
// ulp are truncated: at most one ulp, 2^-52 relative).  A zero or subnormal
// leading part gives 0 (below 2^-126 of the scaled range).
__device__ __forceinline__ double ff_to_double(FF v, int shift) {
    FF n = two_sum(v.s, v.c);
    const uint32_t us = __float_as_uint(n.s), uc = __float_as_uint(n.c);
    const uint32_t ef = us & 0x7f800000u;
    if (ef == 0) return 0.0;
    long long bits = ((long long)(us & 0x7fffffffu) + ((long long)(896 + shift) << 23)) << 29;
    const uint32_t ecf = uc & 0x7f800000u;
    if (ecf != 0) {
        const int sh = 29 - (int)((ef - ecf) >> 23);  // <= 5
        const uint32_t mc = (uc & 0x7fffffu) | 0x800000u;
        const long long add = sh >= 0 ? (long long)(mc << sh) : (sh > -24 ? (long long)(mc >> -sh) : 0);
        bits += ((us ^ uc) >> 31) ? -add : add;
    }
    return __longlong_as_double(bits | ((long long)(us >> 31) << 63));
}

// a 2^Ea + b 2^Eb as one pair with exponent max(Ea, Eb).
__device__ __forceinline__ FF ff_join(FF a, int Ea, bool has_a, FF b, int Eb, bool has_b,
                                      int &E) {
    if (!has_a && !has_b) {
        E = 0;
        return FF{0.f, 0.f};
    }
    if (!has_b) {
        E = Ea;
        return a;
    }
    if (!has_a) {
        E = Eb;
        return b;
    }
    if (Ea < Eb) {
        FF t = a;
        a = b;
        b = t;
        int te = Ea;
        Ea = Eb;
        Eb = te;
    }
    float sc = pow2f(Eb - Ea);
    E = Ea;
    return ff_add(a, FF{__fmul_rn(b.s, sc), __fmul_rn(b.c, sc)});
}

// Minimum resident CTAs per SM the fill kernel is compiled for (caps its
// registers at 65536 / (128 * this)), for the mixed and the FP64 kernel.
// Measured on the order-7, N=200, k=0..10, l_max=5, L=0..3 singlet+triplet
// workload (fill time per step): mixed 8 -> 46.8 ms (64 registers), 7 ->
// 48.9 (72), 6 -> 49.4 (80); FP64 8 -> 28.3 ms, 6 -> 32.1 (80 registers), 10
// -> 35.8 (48, spilling), 12 -> 40.5.  Fewer registers spill in the entry
// loop, more leave too few warps to hide the FP64 and shuffle latencies.
#ifndef BS2E_FILL_MIN_BLOCKS
#define BS2E_FILL_MIN_BLOCKS 8
#endif
#ifndef BS2E_FILL_MIN_BLOCKS_FP64
#define BS2E_FILL_MIN_BLOCKS_FP64 8
#endif
// The large-tile variant (R^k tiles above ~22 KB) is compiled for 4 CTAs per
// SM.  Its FP64 loop takes two entries per lane; measured on four order-9
// N=800 bands (k=0..20, l_max=10; 2.1e9 entries) with the loop written for E
// entries per lane: E=2, 4 CTAs -> 19.7 ms (120 registers); E=4, 4 CTAs ->
// 21.0 (118); E=4, 3 CTAs -> 21.2 (142); E=8, 4 CTAs -> 28.5 (128).  The loop
// is bound by FP64 issue, and a wider group runs more multipole FMAs for
// entries whose sum is then dropped (outside sup or sup_x).  The generic
// form also cost the small-tile kernel 2-3% (more spills), so the two-entry
// loop stays written out.  Cutting rows into units of 8 column channels
// (each unit's offset from the tile's window sums, as the count pass forms
// them) so that a CTA's warps finish together measured 19.93 against 20.04 ms
// on the same bands and 1-1.5% slower on the small tiles: the rows handed out
// largest first already balance the warps, and rows stay the unit.

// Direct + exchange multipole sums of one entry in FP64 from the mixed store
// (each stored pair rescaled exactly to its value), for channel pairs whose
// slice maxima are too far apart for one FP32-pair frame.
__device__ __forceinline__ double wide_sums(const float2 *R2, const int *sexp, const int8_t *kd,
                                            const int8_t *kx, const double *ad, const double *ax,
                                            int nd, int nx, int W2, bool sup, bool supx, int n_c,
                                            int n_d, int n_a, int n_b, int k, int W) {
    double rd = 0.0, rx = 0.0;
    if (sup) {
        const int od = (n_c - n_a + k - 1) * W + (n_d - n_b + k - 1);
        for (int u = 0; u < nd; ++u) {
            const int kk = kd[u];
            const float2 p = R2[kk * W2 + od];
            const double sc = __longlong_as_double((long long)(1023 - kRkBias + sexp[kk]) << 52);
            rd = fma(((double)p.x + (double)p.y) * sc, ad[u], rd);
        }
    }
    if (supx) {
        const int ox = (n_d - n_a + k - 1) * W + (n_c - n_b + k - 1);
        for (int u = 0; u < nx; ++u) {
            const int kk = kx[u];
            const float2 p = R2[kk * W2 + ox];
            const double sc = __longlong_as_double((long long)(1023 - kRkBias + sexp[kk]) << 52);
            rx = fma(((double)p.x + (double)p.y) * sc, ax[u], rx);
        }
    }
    return (sup && supx) ? rd + rx : (sup ? rd : rx);
}

// The rest of one mixed-path H entry once its multipole sums are known: the
// direct (fd, in the frame 2^Ed, present when hd) and exchange (fx, 2^Ex, hx)
// sums are joined, the one-body terms H_1p_neq (mat_els.f90:697-715; od: the
// l_eq term under sup, ox: the l_eq_ex term under sup_x) are added -- as
// FP32 pairs when the bands allow it (ff_one_body), else in FP64 -- and the
// entry is rounded once to a double.  Real S only.  The operations are those
// of the one-entry loop of fill_row, in the same order.
__device__ __forceinline__ double2 mixed_finish(
    const FillArgs &F, FF fd, FF fx, bool hd, bool hx, int Ed, int Ex, bool od, bool ox,
    int n_a, int n_b, int n_c, int n_d, long long sgn_bit, const float4 *HaA, const float4 *HbB,
    const float4 *SA, const float4 *SB, const double2 *HaR, const double2 *HbR,
    const double2 *SaR, const double2 *SbR) {
    int Ev = 0;
    FF v = ff_join(fd, Ed, hd, fx, Ex, hx, Ev);
    bool has = hd || hx;
    double re = 0.0, im = 0.0;
    if (F.ff_one_body) {
        FF hi_im{0.f, 0.f};
        bool fb = false;
        if (od || ox) {
            FF hr{0.f, 0.f};
            if (od) {
                const int dc = n_c - n_a, dd = n_d - n_b;
                float4 h1 = HaA[dc], s1 = SB[dd], h2 = HbB[dd], s2 = SA[dc];
                float2 s1r = make_float2(s1.x, s1.y), s2r = make_float2(s2.x, s2.y);
                hr = ff_add(ff_mul(make_float2(h1.x, h1.y), s1r), ff_mul(make_float2(h2.x, h2.y), s2r));
                hi_im = ff_add(ff_mul(make_float2(h1.z, h1.w), s1r), ff_mul(make_float2(h2.z, h2.w), s2r));
            }
            if (ox) {
                const int dc = n_d - n_a, dd = n_c - n_b;
                float4 h1 = HaA[dc], s1 = SB[dd], h2 = HbB[dd], s2 = SA[dc];
                float2 s1r = make_float2(s1.x, s1.y), s2r = make_float2(s2.x, s2.y);
                const bool ng = sgn_bit != 0;
                FF xr = ff_add(ff_mul(make_float2(h1.x, h1.y), s1r), ff_mul(make_float2(h2.x, h2.y), s2r));
                FF xi = ff_add(ff_mul(make_float2(h1.z, h1.w), s1r), ff_mul(make_float2(h2.z, h2.w), s2r));
                hr = ff_add(hr, ff_neg_if(xr, ng));
                hi_im = ff_add(hi_im, ff_neg_if(xi, ng));
            }
            if (!has || kRkBias - Ev <= 124) {
                v = ff_join(v, Ev, has, hr, kRkBias, true, Ev);
                has = true;
            } else {
                fb = true;
                re = ff_to_double(hr, 0);
            }
        }
        if (has) {
            const double t = ff_to_double(v, Ev - kRkBias);
            re = fb ? re + t : t;
        }
        im = (od || ox) ? ff_to_double(hi_im, 0) : 0.0;
    } else {
        if (has) re = ff_to_double(v, Ev - kRkBias);
        if (od) {
            const int dc = n_c - n_a, dd = n_d - n_b;
            const double2 h1 = HaR[dc], h2 = HbR[dd];
            const double s1 = SbR[dd].x, s2 = SaR[dc].x;
            re = fma(h1.x, s1, re);
            re = fma(h2.x, s2, re);
            im = fma(h1.y, s1, im);
            im = fma(h2.y, s2, im);
        }
        if (ox) {
            const int dc = n_d - n_a, dd = n_c - n_b;
            const double2 h1 = HaR[dc], h2 = HbR[dd];
            const double s1 = flip_sign(SbR[dd].x, sgn_bit);
            const double s2 = flip_sign(SaR[dc].x, sgn_bit);
            re = fma(h1.x, s1, re);
            re = fma(h2.x, s2, re);
            im = fma(h1.y, s1, im);
            im = fma(h2.y, s2, im);
        }
    }
    return make_double2(re, im);
}

// One row of the block (warp-wide): row (n_a, n_b) of channel c_r, with the R^k
// tile of (n_a, n_b) at sR (shared memory when staged, global otherwise), its
// per-multipole exponents at sexp (mixed store) and the warp's scratch for the
// scaled multipole weights.
template <bool MIXED, bool BIG>
__device__ __forceinline__ void fill_row(const FillArgs &F, const int local, const int c_r,
                                         const int n_a, const int n_b, const double *sR,
                                         const int *sexp, float2 (*sAw)[kMaxK1],
                                         int (*sKow)[kMaxK1]) {
    const BlockArgs &A = F.B;
    const float2 *sR2 = (const float2 *)sR;
    const int k = A.k, W = 2 * k - 1, W2 = W * W, K1 = A.K1;
    const int lane = threadIdx.x & 31;
    const unsigned FULL = 0xffffffffu;
    const int l_a = A.chl[c_r] >> 8, l_b = A.chl[c_r] & 255;  // row channel (l1, l2)
    // FP32-pair band rows of this row: X_row[d] = X[n][n+d], |d| < k
    const size_t ra = (size_t)(n_a - 1) * W + (k - 1), rb = (size_t)(n_b - 1) * W + (k - 1);
    const float4 *HaA = F.Hbf ? F.Hbf + (size_t)l_a * A.N * W + ra : nullptr;  // H_la[n_a][.]
    const float4 *HbB = F.Hbf ? F.Hbf + (size_t)l_b * A.N * W + rb : nullptr;  // H_lb[n_b][.]
    const float4 *SA = F.Sbf ? F.Sbf + ra : nullptr;                           // S[n_a][.]
    const float4 *SB = F.Sbf ? F.Sbf + rb : nullptr;                           // S[n_b][.]
    const double2 *HaR = F.Hb + (size_t)l_a * A.N * W + ra;  // FP64 band rows, same indexing
    const double2 *HbR = F.Hb + (size_t)l_b * A.N * W + rb;
    const double2 *SaR = F.Sb + ra, *SbR = F.Sb + rb;
    int64_t oH = F.Hptr[local] - 1 - F.Hbase;
    int64_t oS = F.Sptr[local] - 1 - F.Sbase;
    for (int c_c = A.full ? 0 : c_r; c_c < A.n_ch; ++c_c) {
        const PairInfo pi = A.pairs[(size_t)c_r * A.n_ch + c_c];
        const int flags = pi.flags;
        const bool dir_ok = flags & 1, ex_ok = flags & 2, leq = flags & 4, leqx = flags & 8;
        const bool Aok = dir_ok || leq || leqx, Bok = ex_ok || leq || leqx;
        if (!Aok && !Bok) continue;
        // the exchange sign (+-1) as a sign bit
        const long long sgn_bit = __double_as_longlong(pi.sgn) & (long long)0x8000000000000000ULL;
        const int nlo = (!A.full && c_c == c_r) ? n_a : 1;
        const Iv2 cand = nc_candidates(n_a, n_b, k, A.N, Aok, Bok, nlo);
        const int ncand = cand.l1 + cand.l2;
        const size_t pbase = ((size_t)c_r * A.n_ch + c_c) * 2 * K1;
        const int8_t *kd = A.pair_k + pbase;
        const int8_t *kx = kd + K1;
        const double *ad = A.pair_a + pbase;
        const double *ax = ad + K1;
        int Ed = 0, Ex = 0;
        bool wide = false;
        // FP64: this pair's weights and multipole tile offsets in the warp's
        // shared scratch (the FP32-pair slots), read as broadcasts in the sums
        double (*sAd)[kMaxK1] = reinterpret_cast<double (*)[kMaxK1]>(sAw);
        if (!MIXED) {
            __syncwarp();  // every lane is done with the previous pair's values
            if (lane < pi.nd) {
                sAd[0][lane] = ad[lane];
                sKow[0][lane] = kd[lane] * W2;
            }
            if (lane < pi.nx) {
                sAd[1][lane] = ax[lane];
                sKow[1][lane] = kx[lane] * W2;
            }
            __syncwarp();
        }
        if (MIXED) {
            // scaled multipole weights of this channel pair for this tile
            int ed = -100000, ex = -100000;
            if (lane < pi.nd) ed = sexp[kd[lane]];
            if (lane < pi.nx) ex = sexp[kx[lane]];
            Ed = ed;
            Ex = ex;
            int md = lane < pi.nd ? ed : 100000, mx = lane < pi.nx ? ex : 100000;
            for (int o = 16; o > 0; o >>= 1) {
                Ed = max(Ed, __shfl_xor_sync(FULL, Ed, o));
                Ex = max(Ex, __shfl_xor_sync(FULL, Ex, o));
                md = min(md, __shfl_xor_sync(FULL, md, o));
                mx = min(mx, __shfl_xor_sync(FULL, mx, o));
            }
            // slice maxima more than 2^120 apart: a weight rescaled to the
            // largest would flush while the element of its slice may still
            // matter for an entry, so this pair's sums run in FP64 instead
            // (likewise the direct and exchange frames, which are joined)
            wide = (pi.nd > 0 && Ed - md > 120) || (pi.nx > 0 && Ex - mx > 120) ||
                   (pi.nd > 0 && pi.nx > 0 && abs(Ed - Ex) > 120);
            if (lane < pi.nd) {
                const float *af = A.pair_af + (pbase + lane) * 2;
                float sc = pow2f(ed - Ed);
                sAw[0][lane] = make_float2(__fmul_rn(af[0], sc), __fmul_rn(af[1], sc));
                sKow[0][lane] = kd[lane] * W2;
            }
            if (lane < pi.nx) {
                const float *af = A.pair_af + (pbase + K1 + lane) * 2;
                float sc = pow2f(ex - Ex);
                sAw[1][lane] = make_float2(__fmul_rn(af[0], sc), __fmul_rn(af[1], sc));
                sKow[1][lane] = kx[lane] * W2;
            }
            __syncwarp();
        }
        for (int g0 = 0; g0 < ncand; g0 += 32) {
            const int ci = g0 + lane;
            Iv2 hs{0, 0, 0, 0}, ss{0, 0, 0, 0};
            int base = 0, lo = 0, n_c = 0;
            if (ci < ncand) {
                n_c = iv2_at(cand, ci);
                col_sets(A, c_r, c_c, n_a, n_b, n_c, flags, hs, ss, base, lo);
            }
            // H runs
            {
                int cnt = hs.l1 + hs.l2;
                int incl = cnt;
                for (int o = 1; o < 32; o <<= 1) {
                    int y = __shfl_up_sync(FULL, incl, o);
                    if (lane >= o) incl += y;
                }
                const int excl = incl - cnt;
                const int tot = __shfl_sync(FULL, incl, 31);
                // The reference adds an entry's multipole sums only where
                // r_12_allowed holds (a weight above 5e-15 under sup or sup_x;
                // the sums keep weights above 5e-16).  Unless some pair of the
                // block is flagged (PairInfo bit4: a term whose listed weights
                // are all at most 5e-15; exact 3j/6j values give none),
                // "under sup" alone decides and the two-entry loop needs no
                // per-entry test; a flagged block takes the gated loop below.
                if (!MIXED && F.s_real && !F.gated) {
                    // FP64 with a real S: two entries per lane (e and e + 32 of
                    // each 64), so the two run searches and the two multipole
                    // FMA chains are independent and overlap; an entry outside
                    // sup (sup_x) reads a valid tile element and drops the sum
                    for (int e0 = 0; e0 < tot; e0 += 64) {
                        const int eA = e0 + lane, eB = eA + 32;
                        int pA = 0, pB = 0;
#pragma unroll
                        for (int step = 16; step > 0; step >>= 1) {
                            const int vA = __shfl_sync(FULL, excl, pA + step);
                            const int vB = __shfl_sync(FULL, excl, pB + step);
                            if (vA <= eA) pA += step;
                            if (vB <= eB) pB += step;
                        }
                        int ncA, ndA, jA, ncB, ndB, jB;
                        {
                            const int o = eA - __shfl_sync(FULL, excl, pA);
                            const int l1 = __shfl_sync(FULL, hs.l1, pA);
                            const int s1 = __shfl_sync(FULL, hs.s1, pA), s2 = __shfl_sync(FULL, hs.s2, pA);
                            ncA = __shfl_sync(FULL, n_c, pA);
                            ndA = o < l1 ? s1 + o : s2 + (o - l1);
                            jA = __shfl_sync(FULL, base, pA) + (ndA - __shfl_sync(FULL, lo, pA));
                        }
                        {
                            const int o = eB - __shfl_sync(FULL, excl, pB);
                            const int l1 = __shfl_sync(FULL, hs.l1, pB);
                            const int s1 = __shfl_sync(FULL, hs.s1, pB), s2 = __shfl_sync(FULL, hs.s2, pB);
                            ncB = __shfl_sync(FULL, n_c, pB);
                            ndB = o < l1 ? s1 + o : s2 + (o - l1);
                            jB = __shfl_sync(FULL, base, pB) + (ndB - __shfl_sync(FULL, lo, pB));
                        }
                        const bool liveA = eA < tot, liveB = eB < tot;
                        const bool supA = liveA && abs(n_a - ncA) < k && abs(n_b - ndA) < k;
                        const bool supxA = liveA && abs(n_a - ndA) < k && abs(n_b - ncA) < k;
                        const bool supB = liveB && abs(n_a - ncB) < k && abs(n_b - ndB) < k;
                        const bool supxB = liveB && abs(n_a - ndB) < k && abs(n_b - ncB) < k;
                        double reA = 0.0, imA = 0.0, reB = 0.0, imB = 0.0;
                        if (supA || supB) {
                            const int oA = supA ? (ncA - n_a + k - 1) * W + (ndA - n_b + k - 1) : 0;
                            const int oB = supB ? (ncB - n_a + k - 1) * W + (ndB - n_b + k - 1) : 0;
                            double a = 0.0, b = 0.0;
#pragma unroll 4
                            for (int u = 0; u < pi.nd; ++u) {
                                const int ko = sKow[0][u];
                                const double w = sAd[0][u];
                                a = fma(sR[oA + ko], w, a);
                                b = fma(sR[oB + ko], w, b);
                            }
                            reA = supA ? a : 0.0;
                            reB = supB ? b : 0.0;
                        }
                        if (supxA || supxB) {
                            const int oA = supxA ? (ndA - n_a + k - 1) * W + (ncA - n_b + k - 1) : 0;
                            const int oB = supxB ? (ndB - n_a + k - 1) * W + (ncB - n_b + k - 1) : 0;
                            double a = reA, b = reB;
#pragma unroll 4
                            for (int u = 0; u < pi.nx; ++u) {
                                const int ko = sKow[1][u];
                                const double w = sAd[1][u];
                                a = fma(sR[oA + ko], w, a);
                                b = fma(sR[oB + ko], w, b);
                            }
                            reA = supxA ? a : reA;
                            reB = supxB ? b : reB;
                        }
                        if (leq) {
                            if (supA) {
                                const int dc = ncA - n_a, dd = ndA - n_b;
                                const double2 h1 = HaR[dc], h2 = HbR[dd];
                                const double s1 = SbR[dd].x, s2 = SaR[dc].x;
                                reA = fma(h1.x, s1, reA);
                                reA = fma(h2.x, s2, reA);
                                imA = fma(h1.y, s1, imA);
                                imA = fma(h2.y, s2, imA);
                            }
                            if (supB) {
                                const int dc = ncB - n_a, dd = ndB - n_b;
                                const double2 h1 = HaR[dc], h2 = HbR[dd];
                                const double s1 = SbR[dd].x, s2 = SaR[dc].x;
                                reB = fma(h1.x, s1, reB);
                                reB = fma(h2.x, s2, reB);
                                imB = fma(h1.y, s1, imB);
                                imB = fma(h2.y, s2, imB);
                            }
                        }
                        if (leqx) {
                            if (supxA) {
                                const int dc = ndA - n_a, dd = ncA - n_b;
                                const double2 h1 = HaR[dc], h2 = HbR[dd];
                                const double s1 = flip_sign(SbR[dd].x, sgn_bit), s2 = flip_sign(SaR[dc].x, sgn_bit);
                                reA = fma(h1.x, s1, reA);
                                reA = fma(h2.x, s2, reA);
                                imA = fma(h1.y, s1, imA);
                                imA = fma(h2.y, s2, imA);
                            }
                            if (supxB) {
                                const int dc = ndB - n_a, dd = ncB - n_b;
                                const double2 h1 = HaR[dc], h2 = HbR[dd];
                                const double s1 = flip_sign(SbR[dd].x, sgn_bit), s2 = flip_sign(SaR[dc].x, sgn_bit);
                                reB = fma(h1.x, s1, reB);
                                reB = fma(h2.x, s2, reB);
                                imB = fma(h1.y, s1, imB);
                                imB = fma(h2.y, s2, imB);
                            }
                        }
                        if (liveA) {
                            F.Hidx[oH + eA] = (int64_t)jA + 1;
                            F.Hdat[oH + eA] = make_double2(reA, imA);
                        }
                        if (liveB) {
                            F.Hidx[oH + eB] = (int64_t)jB + 1;
                            F.Hdat[oH + eB] = make_double2(reB, imB);
                        }
                    }
                } else if (MIXED && BIG && F.s_real && !F.gated && !wide) {
                    // mixed path with registers to spare (large-tile variant):
                    // two entries per lane as in the FP64 loop above, so the
                    // FP32-pair accumulations of the two entries form
                    // independent chains; each entry is then finished exactly
                    // as the one-entry loop below does
                    for (int e0 = 0; e0 < tot; e0 += 64) {
                        const int eA = e0 + lane, eB = eA + 32;
                        int pA = 0, pB = 0;
#pragma unroll
                        for (int step = 16; step > 0; step >>= 1) {
                            const int vA = __shfl_sync(FULL, excl, pA + step);
                            const int vB = __shfl_sync(FULL, excl, pB + step);
                            if (vA <= eA) pA += step;
                            if (vB <= eB) pB += step;
                        }
                        int ncA, ndA, jA, ncB, ndB, jB;
                        {
                            const int o = eA - __shfl_sync(FULL, excl, pA);
                            const int l1 = __shfl_sync(FULL, hs.l1, pA);
                            const int s1 = __shfl_sync(FULL, hs.s1, pA), s2 = __shfl_sync(FULL, hs.s2, pA);
                            ncA = __shfl_sync(FULL, n_c, pA);
                            ndA = o < l1 ? s1 + o : s2 + (o - l1);
                            jA = __shfl_sync(FULL, base, pA) + (ndA - __shfl_sync(FULL, lo, pA));
                        }
                        {
                            const int o = eB - __shfl_sync(FULL, excl, pB);
                            const int l1 = __shfl_sync(FULL, hs.l1, pB);
                            const int s1 = __shfl_sync(FULL, hs.s1, pB), s2 = __shfl_sync(FULL, hs.s2, pB);
                            ncB = __shfl_sync(FULL, n_c, pB);
                            ndB = o < l1 ? s1 + o : s2 + (o - l1);
                            jB = __shfl_sync(FULL, base, pB) + (ndB - __shfl_sync(FULL, lo, pB));
                        }
                        const bool liveA = eA < tot, liveB = eB < tot;
                        const bool supA = liveA && abs(n_a - ncA) < k && abs(n_b - ndA) < k;
                        const bool supxA = liveA && abs(n_a - ndA) < k && abs(n_b - ncA) < k;
                        const bool supB = liveB && abs(n_a - ncB) < k && abs(n_b - ndB) < k;
                        const bool supxB = liveB && abs(n_a - ndB) < k && abs(n_b - ncB) < k;
                        // without gated pairs a direct (exchange) sum exists exactly
                        // where sup (sup_x) holds and the list is non-empty
                        const bool hdA = supA && pi.nd > 0, hxA = supxA && pi.nx > 0;
                        const bool hdB = supB && pi.nd > 0, hxB = supxB && pi.nx > 0;
                        FF fdA{0.f, 0.f}, fdB{0.f, 0.f}, fxA{0.f, 0.f}, fxB{0.f, 0.f};
                        if (hdA || hdB) {
                            // an entry without the sum reads a valid element and drops it
                            const int oA = hdA ? (ncA - n_a + k - 1) * W + (ndA - n_b + k - 1) : 0;
                            const int oB = hdB ? (ncB - n_a + k - 1) * W + (ndB - n_b + k - 1) : 0;
#pragma unroll 4
                            for (int u = 0; u < pi.nd; ++u) {
                                const int ko = sKow[0][u];
                                const float2 w = sAw[0][u];
                                ff_madd(fdA, w, sR2[ko + oA]);
                                ff_madd(fdB, w, sR2[ko + oB]);
                            }
                        }
                        if (hxA || hxB) {
                            const int oA = hxA ? (ndA - n_a + k - 1) * W + (ncA - n_b + k - 1) : 0;
                            const int oB = hxB ? (ndB - n_a + k - 1) * W + (ncB - n_b + k - 1) : 0;
#pragma unroll 4
                            for (int u = 0; u < pi.nx; ++u) {
                                const int ko = sKow[1][u];
                                const float2 w = sAw[1][u];
                                ff_madd(fxA, w, sR2[ko + oA]);
                                ff_madd(fxB, w, sR2[ko + oB]);
                            }
                        }
                        if (liveA) {
                            F.Hidx[oH + eA] = (int64_t)jA + 1;
                            F.Hdat[oH + eA] = mixed_finish(F, fdA, fxA, hdA, hxA, Ed, Ex,
                                                           leq && supA, leqx && supxA, n_a, n_b,
                                                           ncA, ndA, sgn_bit, HaA, HbB, SA, SB,
                                                           HaR, HbR, SaR, SbR);
                        }
                        if (liveB) {
                            F.Hidx[oH + eB] = (int64_t)jB + 1;
                            F.Hdat[oH + eB] = mixed_finish(F, fdB, fxB, hdB, hxB, Ed, Ex,
                                                           leq && supB, leqx && supxB, n_a, n_b,
                                                           ncB, ndB, sgn_bit, HaA, HbB, SA, SB,
                                                           HaR, HbR, SaR, SbR);
                        }
                    }
                } else {
                    for (int e0 = 0; e0 < tot; e0 += 32) {
                        const int e = e0 + lane;
                        int pos = 0;
#pragma unroll
                        for (int step = 16; step > 0; step >>= 1) {
                            int cand_pos = pos + step;
                            int v = __shfl_sync(FULL, excl, cand_pos);
                            if (v <= e) pos = cand_pos;
                        }
                        const int o_ex = __shfl_sync(FULL, excl, pos);
                        const int r_nc = __shfl_sync(FULL, n_c, pos);
                        const int r_base = __shfl_sync(FULL, base, pos);
                        const int r_lo = __shfl_sync(FULL, lo, pos);
                        const int r_s1 = __shfl_sync(FULL, hs.s1, pos);
                        const int r_l1 = __shfl_sync(FULL, hs.l1, pos);
                        const int r_s2 = __shfl_sync(FULL, hs.s2, pos);
                        if (e < tot) {
                            const int o = e - o_ex;
                            const int n_d = o < r_l1 ? r_s1 + o : r_s2 + (o - r_l1);
                            const int j = r_base + (n_d - r_lo);
                            const bool sup = abs(n_a - r_nc) < k && abs(n_b - n_d) < k;
                            const bool supx = abs(n_a - n_d) < k && abs(n_b - r_nc) < k;
                            double re = 0.0, im = 0.0;
                            const bool r12 = (sup && dir_ok) || (supx && ex_ok);
                            const bool one = (sup && leq) || (supx && leqx);
                            if (MIXED && F.ff_one_body) {
                                // everything in FP32-pair arithmetic, one rounding to double
                                FF v{0.f, 0.f};
                                int Ev = 0;
                                bool has = false;
                                double wide_re = 0.0;
                                if (r12 && wide) {
                                    wide_re = wide_sums(sR2, sexp, kd, kx, ad, ax, pi.nd, pi.nx, W2,
                                                        sup, supx, r_nc, n_d, n_a, n_b, k, W);
                                } else if (r12) {
                                    const int od = (r_nc - n_a + k - 1) * W + (n_d - n_b + k - 1);
                                    const int ox = (n_d - n_a + k - 1) * W + (r_nc - n_b + k - 1);
                                    FF fd{0.f, 0.f}, fx{0.f, 0.f};
                                    if (sup)
#pragma unroll 4
                                        for (int u = 0; u < pi.nd; ++u)
                                            ff_madd(fd, sAw[0][u], sR2[sKow[0][u] + od]);
                                    if (supx)
#pragma unroll 4
                                        for (int u = 0; u < pi.nx; ++u)
                                            ff_madd(fx, sAw[1][u], sR2[sKow[1][u] + ox]);
                                    v = ff_join(fd, Ed, sup && pi.nd > 0, fx, Ex, supx && pi.nx > 0, Ev);
                                    has = (sup && pi.nd > 0) || (supx && pi.nx > 0);
                                }
                                FF hi_im{0.f, 0.f};
                                bool fb = false;
                                if (one) {
                                    // H_1p_neq (mat_els.f90:697-715) with real S: the l_eq
                                    // term is non-zero only under sup, the l_eq_ex term only
                                    // under sup_x, so both lookups stay inside the band
                                    FF hr{0.f, 0.f};
                                    if (leq && sup) {
                                        const int dc = r_nc - n_a, dd = n_d - n_b;
                                        float4 h1 = HaA[dc], s1 = SB[dd], h2 = HbB[dd], s2 = SA[dc];
                                        float2 s1r = make_float2(s1.x, s1.y), s2r = make_float2(s2.x, s2.y);
                                        hr = ff_add(ff_mul(make_float2(h1.x, h1.y), s1r),
                                                    ff_mul(make_float2(h2.x, h2.y), s2r));
                                        hi_im = ff_add(ff_mul(make_float2(h1.z, h1.w), s1r),
                                                       ff_mul(make_float2(h2.z, h2.w), s2r));
                                    }
                                    if (leqx && supx) {
                                        const int dc = n_d - n_a, dd = r_nc - n_b;
                                        float4 h1 = HaA[dc], s1 = SB[dd], h2 = HbB[dd], s2 = SA[dc];
                                        float2 s1r = make_float2(s1.x, s1.y), s2r = make_float2(s2.x, s2.y);
                                        const bool ng = sgn_bit != 0;
                                        FF xr = ff_add(ff_mul(make_float2(h1.x, h1.y), s1r),
                                                       ff_mul(make_float2(h2.x, h2.y), s2r));
                                        FF xi = ff_add(ff_mul(make_float2(h1.z, h1.w), s1r),
                                                       ff_mul(make_float2(h2.z, h2.w), s2r));
                                        hr = ff_add(hr, ff_neg_if(xr, ng));
                                        hi_im = ff_add(hi_im, ff_neg_if(xi, ng));
                                    }
                                    // the one-body part is in absolute scale (exponent
                                    // kRkBias in the pair's frame), the two-electron part
                                    // in its slice's frame Ev: joined as FP32 pairs while
                                    // the factor 2^(Ev - kRkBias) that rescales the latter
                                    // is a normal float with margin (slice maxima above
                                    // 2^-12, radii below ~4000 a.u., for kRkBias = 112),
                                    // in FP64 otherwise
                                    if (!has || kRkBias - Ev <= 124) {
                                        v = ff_join(v, Ev, has, hr, kRkBias, true, Ev);
                                        has = true;
                                    } else {
                                        fb = true;
                                        re = ff_to_double(hr, 0);
                                    }
                                }
                                if (has) {
                                    const double t = ff_to_double(v, Ev - kRkBias);
                                    if (fb) re = re + t;
                                    else re = t;
                                }
                                if (wide) re = re + wide_re;
                                im = one ? ff_to_double(hi_im, 0) : 0.0;
                            } else if (r12) {
                                const int od = (r_nc - n_a + k - 1) * W + (n_d - n_b + k - 1);
                                const int ox = (n_d - n_a + k - 1) * W + (r_nc - n_b + k - 1);
                                if (MIXED && wide) {
                                    re = wide_sums(sR2, sexp, kd, kx, ad, ax, pi.nd, pi.nx, W2, sup,
                                                   supx, r_nc, n_d, n_a, n_b, k, W);
                                } else if (MIXED) {
                                    FF fd{0.f, 0.f}, fx{0.f, 0.f};
                                    if (sup)
#pragma unroll 4
                                        for (int u = 0; u < pi.nd; ++u)
                                            ff_madd(fd, sAw[0][u], sR2[sKow[0][u] + od]);
                                    if (supx)
#pragma unroll 4
                                        for (int u = 0; u < pi.nx; ++u)
                                            ff_madd(fx, sAw[1][u], sR2[sKow[1][u] + ox]);
                                    int Ev;
                                    FF v = ff_join(fd, Ed, sup && pi.nd > 0, fx, Ex, supx && pi.nx > 0, Ev);
                                    re = ff_to_double(v, Ev - kRkBias);
                                } else {
                                    // direct and exchange multipole sums in one accumulator
                                    // (no FP64 add joins them)
                                    if (sup) {
                                        const double *Rt = sR + od;
                                        for (int u = 0; u < pi.nd; ++u) re = fma(Rt[sKow[0][u]], sAd[0][u], re);
                                    }
                                    if (supx) {
                                        const double *Rt = sR + ox;
                                        for (int u = 0; u < pi.nx; ++u) re = fma(Rt[sKow[1][u]], sAd[1][u], re);
                                    }
                                }
                            }
                            if (one && !(MIXED && F.ff_one_body) && F.s_real) {
                                // H_1p_neq (mat_els.f90:697-715) with a real S: the l_eq
                                // term is non-zero only under sup, the l_eq_ex term only
                                // under sup_x (both lookups inside the band); its
                                // products go straight into the entry's accumulators
                                // and the exchange sign flips the S factors
                                if (leq && sup) {
                                    const int dc = r_nc - n_a, dd = n_d - n_b;
                                    const double2 h1 = HaR[dc], h2 = HbR[dd];
                                    const double s1 = SbR[dd].x, s2 = SaR[dc].x;
                                    re = fma(h1.x, s1, re);
                                    re = fma(h2.x, s2, re);
                                    im = fma(h1.y, s1, im);
                                    im = fma(h2.y, s2, im);
                                }
                                if (leqx && supx) {
                                    const int dc = n_d - n_a, dd = r_nc - n_b;
                                    const double2 h1 = HaR[dc], h2 = HbR[dd];
                                    const double s1 = flip_sign(SbR[dd].x, sgn_bit);
                                    const double s2 = flip_sign(SaR[dc].x, sgn_bit);
                                    re = fma(h1.x, s1, re);
                                    re = fma(h2.x, s2, re);
                                    im = fma(h1.y, s1, im);
                                    im = fma(h2.y, s2, im);
                                }
                            } else if (one && !(MIXED && F.ff_one_body)) {
                                // H_1p_neq (mat_els.f90:697-715), complex S
                                const int N = A.N;
                                const double2 *Ha = F.Hb + (size_t)l_a * N * W;
                                const double2 *Hbb = F.Hb + (size_t)l_b * N * W;
                                double2 h1 = make_double2(0.0, 0.0);
                                if (leq) {
                                    double2 t1 = cmul(band(Ha, N, k, n_a, r_nc), band(F.Sb, N, k, n_b, n_d));
                                    double2 t2 = cmul(band(Hbb, N, k, n_b, n_d), band(F.Sb, N, k, n_a, r_nc));
                                    h1 = cadd(cadd(h1, t1), t2);
                                }
                                if (leqx) {
                                    double2 t1 = cmul(band(Ha, N, k, n_a, n_d), band(F.Sb, N, k, n_b, r_nc));
                                    double2 t2 = cmul(band(Hbb, N, k, n_b, r_nc), band(F.Sb, N, k, n_a, n_d));
                                    double2 t12 = cadd(t1, t2);
                                    h1 = cadd(h1, make_double2(t12.x * pi.sgn, t12.y * pi.sgn));
                                }
                                re = re + h1.x;
                                im = im + h1.y;
                            }
                            F.Hidx[oH + e] = (int64_t)j + 1;
                            F.Hdat[oH + e] = make_double2(re, im);
                        }
                    }
                }
                oH += tot;
            }
            // S runs
            if (leq || leqx) {
                int cnt = ss.l1 + ss.l2;
                int incl = cnt;
                for (int o = 1; o < 32; o <<= 1) {
                    int y = __shfl_up_sync(FULL, incl, o);
                    if (lane >= o) incl += y;
                }
                const int excl = incl - cnt;
                const int tot = __shfl_sync(FULL, incl, 31);
                for (int e0 = 0; e0 < tot; e0 += 32) {
                    const int e = e0 + lane;
                    int pos = 0;
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1) {
                        int cand_pos = pos + step;
                        int v = __shfl_sync(FULL, excl, cand_pos);
                        if (v <= e) pos = cand_pos;
                    }
                    const int o_ex = __shfl_sync(FULL, excl, pos);
                    const int r_nc = __shfl_sync(FULL, n_c, pos);
                    const int r_base = __shfl_sync(FULL, base, pos);
                    const int r_lo = __shfl_sync(FULL, lo, pos);
                    const int r_s1 = __shfl_sync(FULL, ss.s1, pos);
                    const int r_l1 = __shfl_sync(FULL, ss.l1, pos);
                    const int r_s2 = __shfl_sync(FULL, ss.s2, pos);
                    if (e < tot) {
                        const int o = e - o_ex;
                        const int n_d = o < r_l1 ? r_s1 + o : r_s2 + (o - r_l1);
                        const int j = r_base + (n_d - r_lo);
                        // S_mat_neq (mat_els.f90:664-678)
                        const int N = A.N;
                        double2 s1 = make_double2(0.0, 0.0);
                        if (MIXED && F.ff_one_body) {
                            FF t{0.f, 0.f};
                            const bool sup = abs(n_a - r_nc) < k && abs(n_b - n_d) < k;
                            const bool supx = abs(n_a - n_d) < k && abs(n_b - r_nc) < k;
                            if (leq && sup) {
                                float4 a = SA[r_nc - n_a], b = SB[n_d - n_b];
                                t = ff_mul(make_float2(a.x, a.y), make_float2(b.x, b.y));
                            }
                            if (leqx && supx) {
                                float4 a = SA[n_d - n_a], b = SB[r_nc - n_b];
                                t = ff_add(t, ff_neg_if(ff_mul(make_float2(a.x, a.y), make_float2(b.x, b.y)),
                                                        sgn_bit != 0));
                            }
                            s1 = make_double2(ff_to_double(t, 0), 0.0);
                        } else if (F.s_real) {
                            // real S: the l_eq term lives under sup, l_eq_ex under sup_x
                            const bool sup = abs(n_a - r_nc) < k && abs(n_b - n_d) < k;
                            const bool supx = abs(n_a - n_d) < k && abs(n_b - r_nc) < k;
                            double sr = 0.0;
                            if (leq && sup) sr = SaR[r_nc - n_a].x * SbR[n_d - n_b].x;
                            if (leqx && supx)
                                sr = fma(flip_sign(SaR[n_d - n_a].x, sgn_bit), SbR[r_nc - n_b].x, sr);
                            s1 = make_double2(sr, 0.0);
                        } else {
                            if (leq) s1 = cadd(s1, cmul(band(F.Sb, N, k, n_a, r_nc), band(F.Sb, N, k, n_b, n_d)));
                            if (leqx) {
                                double2 a = band(F.Sb, N, k, n_a, n_d);
                                a = make_double2(a.x * pi.sgn, a.y * pi.sgn);
                                s1 = cadd(s1, cmul(a, band(F.Sb, N, k, n_b, r_nc)));
                            }
                        }
                        F.Sidx[oS + e] = (int64_t)j + 1;
                        F.Sdat[oS + e] = s1;
                    }
                }
                oS += tot;
            }
        }
    }
}

// BIG: the variant for R^k tiles too large for 8 CTAs per SM (above ~22 KB:
// order 9 with k <= 20 stages 48.5 KB), compiled for 4 CTAs per SM.  Warps
// per CTA: the FP64 kernel's loop is bound by FP64 issue, and more warps keep
// the pipe fed while others find their entries.  Four order-9 N=800 bands
// (2.1e9 entries) took 19.6 ms with 4 warps (120 registers), 19.2 with 5
// (96), 18.0-18.6 with 6 (80) and 18.1-18.2 with 7 (72, no spills); 7 is the
// most whose shared memory fits four CTAs on an SM (four of 48.5 KB tile +
// 8 KB static + 1 KB reserved).  The mixed kernel needs its 128 registers.
template <bool MIXED, bool BIG>
__host__ __device__ constexpr int fill_warps() { return BIG && !MIXED ? 7 : 4; }

template <bool MIXED, bool BIG>
__global__ void __launch_bounds__(32 * fill_warps<MIXED, BIG>(), BIG ? 4 : (MIXED ? BS2E_FILL_MIN_BLOCKS : BS2E_FILL_MIN_BLOCKS_FP64)) k_csr_fill(FillArgs F) {
    extern __shared__ __align__(128) double sR[];
    __shared__ uint64_t bar;
    __shared__ int sexp[kMaxK1];
    __shared__ float2 sA[fill_warps<MIXED, BIG>()][2][kMaxK1];
    __shared__ int sKo[fill_warps<MIXED, BIG>()][2][kMaxK1];
    __shared__ int srow[kMaxCh], snrow, snext;
    __shared__ uint8_t sch[kMaxCh];
    __shared__ int snz[kMaxCh];
    __shared__ uint8_t sord[kMaxCh];
    static_assert(kMaxCh <= 256, "row order kept in bytes");
    const BlockArgs &A = F.B;
    const int n_a = F.a0 + (int)(blockIdx.x / A.N), n_b = blockIdx.x % A.N + 1;
    const size_t tix = (size_t)(n_a - 1) * A.N + (n_b - 1);
    // rows of this tile: one per channel whose (n1 = n_a) group holds n2 = n_b;
    // srow keeps each row's output index (its pointer slot)
    if (threadIdx.x == 0) snrow = 0;
    __syncthreads();
    for (int c = F.ch0 + threadIdx.x; c < F.ch1; c += blockDim.x) {
        size_t s = (size_t)c * A.segS + n_a;
        int base = A.seg_base[s], lo = A.seg_lo[s], hi = A.seg_hi[s];
        const int64_t row = base + (n_b - lo);
        if (base >= 0 && lo <= n_b && n_b <= hi && row >= F.row0 && row < F.row1) {
            int local = (int)(row - F.ptr_row0);
            if (F.band) {
                // a row outside the band's list would write past its pointer
                // arrays: skip it and report (error word 2)
                const int64_t loc = (int64_t)F.band[A.n_ch + c] + (row - F.band[c]);
                if (row < F.band[c] || loc >= F.band_rows) {
                    atomicExch(F.err, 2);
                    continue;
                }
                local = (int)loc;
            }
            int slot = atomicAdd(&snrow, 1);
            srow[slot] = local;
            sch[slot] = c;
        }
    }
    __syncthreads();
    const int nrow = snrow;
    if (nrow == 0) return;
    const double *src = MIXED ? (const double *)(F.Rf + tix * F.tile) : F.R + tix * F.tile;
    if (MIXED) {
        for (int i = threadIdx.x; i < A.K1; i += blockDim.x) sexp[i] = F.Rexp[tix * A.K1 + i];
    }
    // rows by descending H entry count (a rank sort), handed out one at a
    // time below, so a warp that finishes early takes the next row instead of
    // idling while the others work through an unequal round-robin share
    for (int i = threadIdx.x; i < nrow; i += blockDim.x) {
        const int64_t n = F.Hptr[srow[i] + 1] - F.Hptr[srow[i]];
        snz[i] = (int)min(n, (int64_t)0x7fffffff);
    }
    if (threadIdx.x == 0) snext = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < nrow; i += blockDim.x) {
        int r = 0;
        for (int j = 0; j < nrow; ++j) r += snz[j] > snz[i] || (snz[j] == snz[i] && j < i);
        sord[r] = (uint8_t)i;
    }
    // (stage_tile begins with a barrier, which orders sord before its use)
    if (!stage_tile(src, sR, (uint32_t)(F.tile * sizeof(double)), &bar, F.err)) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (;;) {
        int rr = 0;
        if (lane == 0) rr = atomicAdd(&snext, 1);
        rr = __shfl_sync(0xffffffffu, rr, 0);
        if (rr >= nrow) break;
        const int i = sord[rr];
        fill_row<MIXED, BIG>(F, srow[i], sch[i], n_a, n_b, sR, sexp, sA[warp], sKo[warp]);
    }
}

// Row mode, for row ranges inside one or two channels, where a tile holds a
// single row of the range: a warp per row, and the row's R^k tile read through
// L1/L2 instead of staged (a staged tile would serve one warp and cap the SM
// at a few CTAs).
template <bool MIXED>
__global__ void __launch_bounds__(128, 6) k_csr_fill_rows(FillArgs F) {
    __shared__ int sexpw[4][kMaxK1];
    __shared__ float2 sA[4][2][kMaxK1];
    __shared__ int sKo[4][2][kMaxK1];
    const BlockArgs &A = F.B;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t row = F.row0 + (int64_t)blockIdx.x * 4 + warp;
    if (row >= F.row1) return;  // whole warp
    const bs2e_config cf = A.cfg[row];
    const int n_a = (int)cf.n1, n_b = (int)cf.n2;
    const int c_r = A.lmap[cf.l1 * kMaxL + cf.l2];
    const size_t tix = (size_t)(n_a - 1) * A.N + (n_b - 1);
    const double *R = MIXED ? (const double *)(F.Rf + tix * F.tile) : F.R + tix * F.tile;
    if (MIXED) {
        for (int i = lane; i < A.K1; i += 32) sexpw[warp][i] = F.Rexp[tix * A.K1 + i];
        __syncwarp();
    }
    fill_row<MIXED, false>(F, (int)(row - F.ptr_row0), c_r, n_a, n_b, R, sexpw[warp], sA[warp],
                    sKo[warp]);
}

__global__ void k_gather_i64(const int64_t *__restrict__ src, const int64_t *__restrict__ idx,
                             int64_t n, int64_t *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = src[idx[i]];
}

// Band-local pointers: local row i lies in the channel c with the largest
// local offset band[n_ch + c] <= i (channels without band rows share their
// successor's offset), at block row band[c] + (i - band[n_ch + c]).
__global__ void k_band_ptr(const int *__restrict__ band, const int64_t *__restrict__ boff,
                           int n_ch, int64_t n_rows, const int64_t *__restrict__ pfxH,
                           const int64_t *__restrict__ pfxS, int64_t *__restrict__ Hptr,
                           int64_t *__restrict__ Sptr, int64_t *__restrict__ rows) {
    __shared__ int soff[kMaxCh];
    for (int c = threadIdx.x; c < n_ch; c += blockDim.x) soff[c] = band[n_ch + c];
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= n_rows;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (i == n_rows) {
            Hptr[i] = boff[n_ch] + 1;
            Sptr[i] = boff[2 * n_ch + 1] + 1;
            continue;
        }
        int lo = 0, hi = n_ch - 1;  // largest c with soff[c] <= i
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (soff[mid] <= i) lo = mid;
            else hi = mid - 1;
        }
        const int c = lo;
        const int64_t first = band[c], row = first + (i - soff[c]);
        Hptr[i] = pfxH[row] - pfxH[first] + boff[c] + 1;
        Sptr[i] = pfxS[row] - pfxS[first] + boff[n_ch + 1 + c] + 1;
        if (rows) rows[i] = row + 1;
    }
}

}  // namespace

static BlockArgs block_args(bs2e_handle *h) {
    BlockArgs A;
    const DevBlock &B = h->blk;
    int S = h->g.N + 2;
    A.cfg = B.cfg;
    A.lmap = B.lmap;
    A.chl = B.chl;
    A.segS = S;
    A.seg_base = B.seg;
    A.seg_lo = B.seg + (size_t)h->plan.n_ch * S;
    A.seg_hi = B.seg + (size_t)2 * h->plan.n_ch * S;
    A.pairs = B.pairs;
    A.pair_k = B.pair_k;
    A.pair_a = B.pair_a;
    A.pair_af = B.pair_af;
    A.n_ch = h->plan.n_ch;
    A.N = h->g.N;
    A.k = h->g.k;
    A.K1 = h->g.K1;
    A.full = (int)h->plan.full;
    A.n_rows = h->plan.n_config;
    return A;
}

static inline unsigned grid_rows(int64_t n) {
    int64_t g = (n + 255) / 256;
    if (g > (int64_t)152 * 32) g = (int64_t)152 * 32;
    return (unsigned)(g < 1 ? 1 : g);
}

void launch_cfg_equal(bs2e_handle *h, const bs2e_config *a, const bs2e_config *b, int64_t n,
                      unsigned long long *stats) {
    if (n <= 0) return;
    k_cfg_equal<<<grid_rows(n), 256, 0, h->stream>>>(a, b, n, stats);
    h->launches++;
}

void launch_chan_marks_on(bs2e_handle *h, const bs2e_config *cfg, int64_t n, int4 *marks, int cap,
                          unsigned long long *stats) {
    if (n <= 0) return;
    k_chan_marks<<<grid_rows(n), 256, 0, h->stream>>>(cfg, n, h->g.N, marks, cap, stats);
    h->launches++;
}

void launch_plan_seg_on(bs2e_handle *h, const bs2e_config *cfg, int64_t n, const int *lmap,
                        int segS, int *base, int *lo, int *hi, unsigned long long *stats) {
    if (n <= 0) return;
    k_plan_seg<<<grid_rows(n), 256, 0, h->stream>>>(cfg, n, lmap, segS, base, lo, hi, stats);
    h->launches++;
}

void launch_chan_marks(bs2e_handle *h, int64_t n) {
    if (n <= 0) return;
    k_chan_marks<<<grid_rows(n), 256, 0, h->stream>>>(h->blk.cfg_new, n, h->g.N, h->blk.marks,
                                                       kMaxCh + 1, h->blk.stats);
    h->launches++;
}

void launch_plan_seg(bs2e_handle *h, int64_t n) {
    if (n <= 0) return;
    BlockArgs A = block_args(h);
    k_plan_seg<<<grid_rows(n), 256, 0, h->stream>>>(h->blk.cfg_new, n, A.lmap, A.segS,
                                                     (int *)A.seg_base, (int *)A.seg_lo,
                                                     (int *)A.seg_hi, h->blk.stats);
    h->launches++;
}

void launch_block_count(bs2e_handle *h) {
    BlockArgs A = block_args(h);
    A.cfg = h->blk.cfg_new;
    int64_t n = h->plan.n_config;
    if (n > 0) {
        const unsigned tiles = (unsigned)((int64_t)A.N * A.N);
        k_csr_count_tiles<<<tiles, 128, 0, h->stream>>>(A, 1, h->blk.cntH, h->blk.cntS,
                                                         h->blk.stats);
        h->launches++;
    }
}

void scan_one(bs2e_handle *h, const int64_t *in, int64_t n, int64_t *part, int64_t *ptr) {
    int64_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb < 1) nb = 1;
    k_scan_partials<<<(unsigned)nb, kScanThreads, 0, h->stream>>>(in, n, part);
    k_scan_part_prefix<<<1, kScanThreads, 0, h->stream>>>(part, nb);
    k_scan_final<<<(unsigned)nb, kScanThreads, 0, h->stream>>>(in, n, part, ptr);
    h->launches += 3;
}

void launch_block_scan(bs2e_handle *h, int64_t *d_Hptr, int64_t *d_Sptr, int64_t row0,
                       int64_t n) {
    int64_t *part = h->blk.scan_tmp;
    scan_one(h, h->blk.cntH + row0, n, part, d_Hptr);
    scan_one(h, h->blk.cntS + row0, n, part, d_Sptr);
}

size_t fill_smem(const Radial &g) { return (size_t)g.tile * sizeof(double); }

void launch_block_fill(bs2e_handle *h, const FillRange &r, const int64_t *d_Hptr,
                       const int64_t *d_Sptr, int64_t *d_Hidx, double2 *d_Hdat, int64_t *d_Sidx,
                       double2 *d_Sdat) {
    FillArgs F;
    F.B = block_args(h);
    F.R = h->d_R;
    F.Rf = h->d_Rf;
    F.Rexp = h->d_Rexp;
    F.tile = h->g.tile;
    F.Hb = h->d_Hb;
    F.Sb = h->d_Sb;
    F.Hbf = h->d_Hbf;
    F.Sbf = h->d_Sbf;
    F.s_real = h->s_real ? 1 : 0;
    F.gated = h->plan.gated ? 1 : 0;
    F.ff_one_body = h->ff_one_body ? 1 : 0;
    F.Hptr = d_Hptr;
    F.Sptr = d_Sptr;
    F.Hidx = d_Hidx;
    F.Sidx = d_Sidx;
    F.Hdat = d_Hdat;
    F.Sdat = d_Sdat;
    F.err = h->d_err;
    F.row0 = r.row0;
    F.row1 = r.row1;
    F.ptr_row0 = r.ptr_row0;
    F.Hbase = r.Hbase;
    F.Sbase = r.Sbase;
    F.a0 = r.a0;
    F.band = r.band;
    F.band_rows = r.band_rows;
    F.ch0 = std::max(r.ch0, 0);
    F.ch1 = r.ch1 < 0 ? F.B.n_ch : std::min(r.ch1, F.B.n_ch);
    size_t smem = fill_smem(h->g);
    if (h->plan.n_config > 0 && r.row1 > r.row0 && r.rows_mode) {
        const unsigned grid = (unsigned)((r.row1 - r.row0 + 3) / 4);
        if (h->precision == BS2E_PREC_MIXED)
            k_csr_fill_rows<true><<<grid, 128, 0, h->stream>>>(F);
        else
            k_csr_fill_rows<false><<<grid, 128, 0, h->stream>>>(F);
        h->launches++;
        return;
    }
    if (h->plan.n_config > 0 && r.row1 > r.row0 && r.a1 >= r.a0) {
        const unsigned tiles = (unsigned)((int64_t)(r.a1 - r.a0 + 1) * h->g.N);
        // 8 CTAs of 128 threads fit an SM while each stages at most ~22 KB
        const bool big = smem > (size_t)22 * 1024;
        auto go = [&](auto kern, int threads) {
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            kern<<<tiles, threads, smem, h->stream>>>(F);
        };
        const bool mixed = h->precision == BS2E_PREC_MIXED;
        if (mixed && big) go(k_csr_fill<true, true>, 32 * fill_warps<true, true>());
        else if (mixed) go(k_csr_fill<true, false>, 32 * fill_warps<true, false>());
        else if (big) go(k_csr_fill<false, true>, 32 * fill_warps<false, true>());
        else go(k_csr_fill<false, false>, 32 * fill_warps<false, false>());
        h->launches++;
    }
}

}  // namespace bs2e

namespace bs2e {

void launch_gather_i64(bs2e_handle *h, const int64_t *src, const int64_t *idx, int64_t n,
                       int64_t *out) {
    if (n <= 0) return;
    k_gather_i64<<<grid_rows(n), 256, 0, h->stream>>>(src, idx, n, out);
    h->launches++;
}

void launch_band_ptr(bs2e_handle *h, const int *band, const int64_t *boff, int n_ch,
                     int64_t n_rows, int64_t *Hptr, int64_t *Sptr, int64_t *rows) {
    k_band_ptr<<<grid_rows(n_rows + 1), 256, 0, h->stream>>>(band, boff, n_ch, n_rows,
                                                             h->blk.pfxH, h->blk.pfxS, Hptr,
                                                             Sptr, rows);
    h->launches++;
}

}  // namespace bs2e
