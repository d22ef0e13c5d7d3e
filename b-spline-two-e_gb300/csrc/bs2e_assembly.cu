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

namespace bs2e {
namespace {

struct Iv2 {  // up to two disjoint ascending integer intervals [s1, s1+l1) and [s2, s2+l2)
    int s1, l1, s2, l2;
};

__device__ __forceinline__ Iv2 make_union(int a0, int a1, bool ina, int b0, int b1, bool inb) {
    // intervals [a0,a1] (if ina, non-empty) and [b0,b1] (if inb)
    Iv2 r{0, 0, 0, 0};
    bool ea = ina && a1 >= a0, eb = inb && b1 >= b0;
    if (ea && eb) {
        if (b0 < a0) {  // order so that a comes first
            int t0 = a0, t1 = a1;
            a0 = b0;
            a1 = b1;
            b0 = t0;
            b1 = t1;
        }
        if (b0 <= a1 + 1) {  // overlap or adjacent: merge
            r.s1 = a0;
            r.l1 = max(a1, b1) - a0 + 1;
        } else {
            r.s1 = a0;
            r.l1 = a1 - a0 + 1;
            r.s2 = b0;
            r.l2 = b1 - b0 + 1;
        }
    } else if (ea) {
        r.s1 = a0;
        r.l1 = a1 - a0 + 1;
    } else if (eb) {
        r.s1 = b0;
        r.l1 = b1 - b0 + 1;
    }
    return r;
}

struct BlockArgs {
    const int4 *rows;
    const int *seg_base, *seg_lo, *seg_hi;  // [n_ch][N+2]
    const PairInfo *pairs;
    const int8_t *pair_k;
    const double *pair_a;
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

// Candidate n_c values of a column channel: union of A (if a_on) and B (if b_on)
// clipped to [nlo, N]; returned as two intervals.
__device__ __forceinline__ Iv2 nc_candidates(int n_a, int n_b, int k, int N, bool a_on, bool b_on,
                                             int nlo) {
    return make_union(max(n_a - k + 1, nlo), min(n_a + k - 1, N), a_on, max(n_b - k + 1, nlo),
                      min(n_b + k - 1, N), b_on);
}

__device__ __forceinline__ int iv2_at(const Iv2 &u, int i) {
    return i < u.l1 ? u.s1 + i : u.s2 + (i - u.l1);
}

// Overlap length of [a0,a1] and [b0,b1].
__device__ __forceinline__ int ovl(int a0, int a1, int b0, int b1) {
    return max(0, min(a1, b1) - max(a0, b0) + 1);
}

// ---------------------------------------------------------------------------
// Count: one thread per row.  cnt_H / cnt_S use the construct predicate; the
// totals of the count_nnz predicate (hamiltonian.f90:386-413) are accumulated
// in ref[0..1] so the host can detect a block where the two disagree.
// ---------------------------------------------------------------------------
__global__ void k_count(BlockArgs A, int64_t *__restrict__ cntH, int64_t *__restrict__ cntS,
                        unsigned long long *__restrict__ ref) {
    int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    long long refH = 0, refS = 0;
    if (row < A.n_rows) {
        int4 rw = A.rows[row];
        int n_a = rw.x, n_b = rw.y, c_r = rw.z;
        const int k = A.k;
        int64_t ch = 0, cs = 0;
        for (int c_c = A.full ? 0 : c_r; c_c < A.n_ch; ++c_c) {
            int flags = A.pairs[(size_t)c_r * A.n_ch + c_c].flags;
            bool dir_ok = flags & 1, ex_ok = flags & 2, leq = flags & 4, leqx = flags & 8;
            int nlo = (!A.full && c_c == c_r) ? n_a : 1;
            Iv2 cand = nc_candidates(n_a, n_b, k, A.N, true, true, nlo);
            int ncand = cand.l1 + cand.l2;
            for (int t = 0; t < ncand; ++t) {
                int n_c = iv2_at(cand, t);
                Iv2 hs, ss;
                int base, lo;
                col_sets(A, c_r, c_c, n_a, n_b, n_c, flags, hs, ss, base, lo);
                ch += hs.l1 + hs.l2;
                cs += ss.l1 + ss.l2;
                // count_nnz semantics: sup entries count if dir_ok, sup_x-only entries if ex_ok
                size_t s = (size_t)c_c * A.segS + n_c;
                int lo2 = A.seg_lo[s], hi = A.seg_hi[s];
                if (A.seg_base[s] < 0) continue;
                if (!A.full && c_c == c_r && n_c == n_a) lo2 = max(lo2, n_b);
                if (hi < lo2) continue;
                bool in_a = abs(n_c - n_a) < k, in_b = abs(n_c - n_b) < k;
                int ysup = in_a ? ovl(n_b - k + 1, n_b + k - 1, lo2, hi) : 0;
                int yx = in_b ? ovl(n_a - k + 1, n_a + k - 1, lo2, hi) : 0;
                int both = (in_a && in_b) ? max(0, min(min(n_b + k - 1, n_a + k - 1), hi) -
                                                      max(max(n_b - k + 1, n_a - k + 1), lo2) + 1)
                                          : 0;
                int xonly = yx - both;
                refH += (dir_ok ? ysup : 0) + (ex_ok ? xonly : 0);
                refS += (leq ? ysup : 0) + (leqx ? xonly : 0);
            }
        }
        cntH[row] = ch;
        cntS[row] = cs;
    }
    // block reduction of the reference counts
    for (int o = 16; o > 0; o >>= 1) {
        refH += __shfl_down_sync(0xffffffffu, refH, o);
        refS += __shfl_down_sync(0xffffffffu, refS, o);
    }
    if ((threadIdx.x & 31) == 0 && (refH || refS)) {
        atomicAdd(&ref[0], (unsigned long long)refH);
        atomicAdd(&ref[1], (unsigned long long)refS);
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
    const int *tile_ab, *tile_ptr, *tile_rows;
    const double *R;
    int64_t tile;
    const double2 *Hb, *Sb;
    int s_real;
    const int64_t *Hptr, *Sptr;  // 1-based CSR pointers of the block
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
    if (d >= k || -d >= k) return make_double2(0.0, 0.0);
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

__global__ void __launch_bounds__(128) k_fill(FillArgs F) {
    extern __shared__ __align__(128) double sR[];
    __shared__ uint64_t bar;
    const BlockArgs &A = F.B;
    const int t = blockIdx.x;
    const int n_a = F.tile_ab[2 * t], n_b = F.tile_ab[2 * t + 1];
    const double *src = F.R + (size_t)((n_a - 1) * A.N + (n_b - 1)) * F.tile;
    if (!stage_tile(src, sR, (uint32_t)(F.tile * sizeof(double)), &bar, F.err)) return;

    const int k = A.k, W = 2 * k - 1, W2 = W * W, K1 = A.K1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const unsigned FULL = 0xffffffffu;
    for (int rr = F.tile_ptr[t] + warp; rr < F.tile_ptr[t + 1]; rr += nwarp) {
        const int row = F.tile_rows[rr];
        const int4 rw = A.rows[row];
        const int c_r = rw.z;
        const int l_a = rw.w >> 8, l_b = rw.w & 255;  // row channel (l1, l2)
        int64_t oH = F.Hptr[row] - 1, oS = F.Sptr[row] - 1;
        for (int c_c = A.full ? 0 : c_r; c_c < A.n_ch; ++c_c) {
            const PairInfo pi = A.pairs[(size_t)c_r * A.n_ch + c_c];
            const int flags = pi.flags;
            const bool dir_ok = flags & 1, ex_ok = flags & 2, leq = flags & 4, leqx = flags & 8;
            const bool Aok = dir_ok || leq || leqx, Bok = ex_ok || leq || leqx;
            if (!Aok && !Bok) continue;
            const int nlo = (!A.full && c_c == c_r) ? n_a : 1;
            const Iv2 cand = nc_candidates(n_a, n_b, k, A.N, Aok, Bok, nlo);
            const int ncand = cand.l1 + cand.l2;
            const size_t pbase = ((size_t)c_r * A.n_ch + c_c) * 2 * K1;
            const int8_t *kd = A.pair_k + pbase;
            const int8_t *kx = kd + K1;
            const double *ad = A.pair_a + pbase;
            const double *ax = ad + K1;
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
                            if ((sup && dir_ok) || (supx && ex_ok)) {
                                double res = 0.0;
                                if (sup) {
                                    const double *Rt = sR + (r_nc - n_a + k - 1) * W + (n_d - n_b + k - 1);
                                    double r = 0.0;
                                    for (int u = 0; u < pi.nd; ++u) r = fma(Rt[kd[u] * W2], ad[u], r);
                                    res = res + r;
                                }
                                if (supx) {
                                    const double *Rt = sR + (n_d - n_a + k - 1) * W + (r_nc - n_b + k - 1);
                                    double r = 0.0;
                                    for (int u = 0; u < pi.nx; ++u) r = fma(Rt[kx[u] * W2], ax[u], r);
                                    res = res + r;
                                }
                                re = res;
                            }
                            if ((sup && leq) || (supx && leqx)) {
                                // H_1p_neq (mat_els.f90:697-715)
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
                            if (leq) s1 = cadd(s1, cmul(band(F.Sb, N, k, n_a, r_nc), band(F.Sb, N, k, n_b, n_d)));
                            if (leqx) {
                                double2 a = band(F.Sb, N, k, n_a, n_d);
                                a = make_double2(a.x * pi.sgn, a.y * pi.sgn);
                                s1 = cadd(s1, cmul(a, band(F.Sb, N, k, n_b, r_nc)));
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
}

}  // namespace

static BlockArgs block_args(bs2e_handle *h) {
    BlockArgs A;
    A.rows = h->blk.rows;
    int S = h->g.N + 2;
    A.segS = S;
    A.seg_base = h->blk.seg;
    A.seg_lo = h->blk.seg + (size_t)h->plan.n_ch * S;
    A.seg_hi = h->blk.seg + (size_t)2 * h->plan.n_ch * S;
    A.pairs = h->blk.pairs;
    A.pair_k = h->blk.pair_k;
    A.pair_a = h->blk.pair_a;
    A.n_ch = h->plan.n_ch;
    A.N = h->g.N;
    A.k = h->g.k;
    A.K1 = h->g.K1;
    A.full = (int)h->plan.full;
    A.n_rows = h->plan.n_config;
    return A;
}

void launch_block_count(bs2e_handle *h) {
    BlockArgs A = block_args(h);
    int64_t n = h->plan.n_config;
    unsigned long long *ref = (unsigned long long *)h->blk.scan_tmp;  // first two words
    cudaMemsetAsync(ref, 0, 2 * sizeof(unsigned long long), h->stream);
    if (n > 0) {
        k_count<<<(unsigned)((n + 127) / 128), 128, 0, h->stream>>>(A, h->blk.cntH, h->blk.cntS, ref);
        h->launches++;
    }
}

static void scan_one(bs2e_handle *h, const int64_t *in, int64_t n, int64_t *part, int64_t *ptr) {
    int64_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb < 1) nb = 1;
    k_scan_partials<<<(unsigned)nb, kScanThreads, 0, h->stream>>>(in, n, part);
    k_scan_part_prefix<<<1, kScanThreads, 0, h->stream>>>(part, nb);
    k_scan_final<<<(unsigned)nb, kScanThreads, 0, h->stream>>>(in, n, part, ptr);
    h->launches += 3;
}

void launch_block_scan(bs2e_handle *h, int64_t *d_Hptr, int64_t *d_Sptr) {
    int64_t n = h->plan.n_config;
    int64_t *part = h->blk.scan_tmp + 2;
    scan_one(h, h->blk.cntH, n, part, d_Hptr);
    scan_one(h, h->blk.cntS, n, part, d_Sptr);
}

size_t fill_smem(const Radial &g) { return (size_t)g.tile * sizeof(double); }

void launch_block_fill(bs2e_handle *h, const int64_t *d_Hptr, const int64_t *d_Sptr,
                       int64_t *d_Hidx, double2 *d_Hdat, int64_t *d_Sidx, double2 *d_Sdat) {
    FillArgs F;
    F.B = block_args(h);
    F.tile_ab = h->blk.tile_ab;
    F.tile_ptr = h->blk.tile_ptr;
    F.tile_rows = h->blk.tile_rows;
    F.R = h->d_R;
    F.tile = h->g.tile;
    F.Hb = h->d_Hb;
    F.Sb = h->d_Sb;
    F.s_real = h->s_real ? 1 : 0;
    F.Hptr = d_Hptr;
    F.Sptr = d_Sptr;
    F.Hidx = d_Hidx;
    F.Sidx = d_Sidx;
    F.Hdat = d_Hdat;
    F.Sdat = d_Sdat;
    F.err = h->d_err;
    size_t smem = fill_smem(h->g);
    cudaFuncSetAttribute(k_fill, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (h->blk.n_tiles > 0) {
        k_fill<<<(unsigned)h->blk.n_tiles, 128, smem, h->stream>>>(F);
        h->launches++;
    }
}

}  // namespace bs2e
