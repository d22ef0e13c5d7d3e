// bs2e_dipole.cu -- dipole couplings between symmetry blocks.
//
// Reference: setup_radial_dip / compute_radial_dip_len / _vel
// (src/mat_els/mat_els.f90:120-170, 348-390), dip_mat_neq, dip_red_mat,
// dip_red_1p_len / _vel, ang_dip_red (mat_els.f90:717-829), and
// construct_dip_block_tensor with init_dip_block (src/mat_els/dipole.f90:8-146).
//
// For a row configuration (n_a, n_b; l_a, l_b) of symmetry 1 and a column
// configuration (n_c, n_d; l_c, l_d) of symmetry 2 the entry is stored when
// (sup or sup_x) and ang_dip_red(L1, L2, confs) > 5e-16, with sup / sup_x as
// for H; its value is
//   ang3j [ c1 m1(n_a,n_c) S(n_b,n_d) + c2 m2(n_b,n_d) S(n_a,n_c)
//         + c1x m1x(n_a,n_d) S(n_b,n_c) + c2x m2x(n_b,n_c) S(n_a,n_d) ]
// where m = alpha M1 + beta M2 is the one-particle reduced dipole (length
// gauge: M1 = <r>, velocity: M1 = <-i d/dr>, M2 = <-i/r>) and the c's carry the
// 6j, the sqrt((2L1+1)(2L2+1)) factor and the phases; the channel-pair
// coefficients are computed on the host.
#include <cuda_runtime.h>

#include "bs2e_device.cuh"
#include "bs2e_internal.h"

namespace bs2e {
namespace {

__device__ __forceinline__ double2 bnd(const double2 *M, int k, int x, int y) {
    int d = y - x;
    if (M == nullptr || abs(d) >= k) return make_double2(0.0, 0.0);
    return M[(size_t)(x - 1) * (2 * k - 1) + (d + k - 1)];
}
__device__ __forceinline__ double2 cmul2(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// (a M1 + b M2)(x, y) * S(u, v); the caller skips terms whose a and b are
// both zero
__device__ __forceinline__ double2 dterm(double a, double b, const double2 *M1, const double2 *M2,
                                         const double2 *Sb, int k, int x, int y, int u, int v) {
    double2 m1 = bnd(M1, k, x, y), m2 = bnd(M2, k, x, y);
    double2 m = make_double2(a * m1.x + b * m2.x, a * m1.y + b * m2.y);
    return cmul2(m, bnd(Sb, k, u, v));
}

struct DipArgs {
    const bs2e_config *rows;
    int64_t n_rows;
    const int *lmap_r;                      // row (l1, l2) -> row channel
    const int *seg_base, *seg_lo, *seg_hi;  // column segment tables [n_ch_c][N+2]
    int segS, n_ch_r, n_ch_c, N, k;
    const DipPair *pairs;  // [n_ch_r][n_ch_c]
    const double2 *M1, *M2, *Sb;
};

__device__ __forceinline__ Iv2 dip_cols(const DipArgs &A, int cc, int n_a, int n_b, int n_c,
                                        int &base, int &lo) {
    const int k = A.k;
    size_t s = (size_t)cc * A.segS + n_c;
    base = A.seg_base[s];
    lo = A.seg_lo[s];
    int hi = A.seg_hi[s];
    if (base < 0 || hi < lo) return Iv2{0, 0, 0, 0};
    bool in_a = abs(n_c - n_a) < k, in_b = abs(n_c - n_b) < k;
    return make_union(max(n_b - k + 1, lo), min(n_b + k - 1, hi), in_a, max(n_a - k + 1, lo),
                      min(n_a + k - 1, hi), in_b);
}

__global__ void k_dip_count(DipArgs A, int64_t *__restrict__ cnt,
                            unsigned long long *__restrict__ stats) {
    int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    long long tot = 0;
    if (row < A.n_rows) {
        const bs2e_config cf = A.rows[row];
        const int n_a = (int)cf.n1, n_b = (int)cf.n2;
        const int cr = A.lmap_r[cf.l1 * kMaxL + cf.l2];
        for (int cc = 0; cc < A.n_ch_c; ++cc) {
            if (!A.pairs[(size_t)cr * A.n_ch_c + cc].ok) continue;
            Iv2 cand = nc_candidates(n_a, n_b, A.k, A.N, true, true, 1);
            for (int t = 0; t < cand.l1 + cand.l2; ++t) {
                int base, lo;
                Iv2 u = dip_cols(A, cc, n_a, n_b, iv2_at(cand, t), base, lo);
                tot += u.l1 + u.l2;
            }
        }
        cnt[row] = tot;
    }
    for (int o = 16; o > 0; o >>= 1) tot += __shfl_down_sync(0xffffffffu, tot, o);
    if ((threadIdx.x & 31) == 0 && tot) atomicAdd(&stats[3], (unsigned long long)tot);
}

// The entry value in real arithmetic when S and the radial dipole bands are
// real (P = 0: the value is real) or S real and the bands imaginary (P = 1:
// the value is imaginary, the imaginary parts carry it): one product-sum per
// term instead of a complex one.  The caller skips terms whose a and b are
// both zero.
template <int P>
__device__ __forceinline__ double dterm_part(double a, double b, const double *M1, const double *M2,
                                             const double *S, int k, int x, int y, int u, int v,
                                             double acc) {
    const int W = 2 * k - 1;
    const int d = y - x, e = v - u;
    // (written with abs: the equivalent test `d >= k || -d >= k || e >= k ||
    // -e >= k` came out wrong for some inputs in this function on sm_103a,
    // checked against a CPU reference over all (x, y, u, v) of a 24-spline
    // grid; the abs form and an unsigned range test were exact)
    if (abs(d) >= k || abs(e) >= k) return acc;
    const size_t om = (size_t)(x - 1) * W + (d + k - 1), os = (size_t)(u - 1) * W + (e + k - 1);
    const double m = a * M1[2 * om + P] + (M2 ? b * M2[2 * om + P] : 0.0);
    return fma(m, S[2 * os], acc);
}

// One warp per row; lanes enumerate the (n_c, n_d) runs of each column channel
// exactly as the H assembly does, so columns come out ascending.  MODE 0:
// complex arithmetic; 1: S and the dipole bands real; 2: S real, the bands
// imaginary (the radial dipoles the library computes are one or the other).
template <int MODE>
__global__ void __launch_bounds__(128) k_dip_fill(DipArgs A, const int64_t *__restrict__ ptr,
                                                  int64_t *__restrict__ idx,
                                                  double2 *__restrict__ dat) {
    const int lane = threadIdx.x & 31;
    const unsigned FULL = 0xffffffffu;
    const int64_t row = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= A.n_rows) return;
    const bs2e_config cf = A.rows[row];
    const int n_a = (int)cf.n1, n_b = (int)cf.n2, k = A.k;
    const int cr = A.lmap_r[cf.l1 * kMaxL + cf.l2];
    int64_t o_row = ptr[row] - 1;
    for (int cc = 0; cc < A.n_ch_c; ++cc) {
        const DipPair pp = A.pairs[(size_t)cr * A.n_ch_c + cc];
        if (!pp.ok) continue;
        // which of the four terms have a non-zero coefficient pair, decided
        // on the host: a double comparison runs on GB300's FP64 pipe, and the
        // eight of them per channel pair, on rows of ~50 entries per pair,
        // kept that pipe 82% busy while the entries' own products used 11%
        // of it (order-9 N=200 slice of the L=4 -> 5 block, 181e6 entries)
        const int tm = pp.tm;
        const Iv2 cand = nc_candidates(n_a, n_b, k, A.N, true, true, 1);
        const int ncand = cand.l1 + cand.l2;
        for (int g0 = 0; g0 < ncand; g0 += 32) {
            const int ci = g0 + lane;
            Iv2 run{0, 0, 0, 0};
            int base = 0, lo = 0, n_c = 0;
            if (ci < ncand) {
                n_c = iv2_at(cand, ci);
                run = dip_cols(A, cc, n_a, n_b, n_c, base, lo);
            }
            int cnt = run.l1 + run.l2, incl = cnt;
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
                    int cp = pos + step;
                    if (__shfl_sync(FULL, excl, cp) <= e) pos = cp;
                }
                const int o_ex = __shfl_sync(FULL, excl, pos);
                const int r_nc = __shfl_sync(FULL, n_c, pos);
                const int r_base = __shfl_sync(FULL, base, pos);
                const int r_lo = __shfl_sync(FULL, lo, pos);
                const int r_s1 = __shfl_sync(FULL, run.s1, pos);
                const int r_l1 = __shfl_sync(FULL, run.l1, pos);
                const int r_s2 = __shfl_sync(FULL, run.s2, pos);
                if (e < tot) {
                    const int o = e - o_ex;
                    const int n_d = o < r_l1 ? r_s1 + o : r_s2 + (o - r_l1);
                    double2 v;
                    if (MODE == 0) {
                        const double2 z = make_double2(0.0, 0.0);
                        v = (tm & 1) ? dterm(pp.c[0], pp.c[1], A.M1, A.M2, A.Sb, k, n_a, r_nc, n_b, n_d) : z;
                        double2 t = (tm & 2) ? dterm(pp.c[2], pp.c[3], A.M1, A.M2, A.Sb, k, n_b, n_d, n_a, r_nc) : z;
                        v = make_double2(v.x + t.x, v.y + t.y);
                        t = (tm & 4) ? dterm(pp.c[4], pp.c[5], A.M1, A.M2, A.Sb, k, n_a, n_d, n_b, r_nc) : z;
                        v = make_double2(v.x + t.x, v.y + t.y);
                        t = (tm & 8) ? dterm(pp.c[6], pp.c[7], A.M1, A.M2, A.Sb, k, n_b, r_nc, n_a, n_d) : z;
                        v = make_double2(v.x + t.x, v.y + t.y);
                    } else {
                        constexpr int P = MODE == 1 ? 0 : 1;
                        const double *M1 = (const double *)A.M1, *M2 = (const double *)A.M2;
                        const double *S = (const double *)A.Sb;
                        double s = 0.0;
                        if (tm & 1) s = dterm_part<P>(pp.c[0], pp.c[1], M1, M2, S, k, n_a, r_nc, n_b, n_d, s);
                        if (tm & 2) s = dterm_part<P>(pp.c[2], pp.c[3], M1, M2, S, k, n_b, n_d, n_a, r_nc, s);
                        if (tm & 4) s = dterm_part<P>(pp.c[4], pp.c[5], M1, M2, S, k, n_a, n_d, n_b, r_nc, s);
                        if (tm & 8) s = dterm_part<P>(pp.c[6], pp.c[7], M1, M2, S, k, n_b, r_nc, n_a, n_d, s);
                        v = MODE == 1 ? make_double2(s, 0.0) : make_double2(0.0, s);
                    }
                    idx[o_row + e] = (int64_t)(r_base + (n_d - r_lo)) + 1;
                    dat[o_row + e] = v;
                }
            }
            o_row += tot;
        }
    }
}

// Radial dipole bands from the tabulated spline values and first derivatives:
//   gauge 0: M1 = sum w r B_i B_j                   (compute_radial_dip_len)
//   gauge 1: M1 = -i sum w B_i B_j', M2 = -i sum w B_i B_j / r   (compute_radial_dip_vel)
__global__ void k_radial_dip(const double *__restrict__ knots, const double *__restrict__ glw,
                             const double *__restrict__ tab_r, const double *__restrict__ tab_B,
                             const double *__restrict__ tab_D1, int k, int q, int N, int n_iv,
                             int gauge, double2 *__restrict__ M1, double2 *__restrict__ M2) {
    const int W = 2 * k - 1;
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= N * W) return;
    int i = e / W, j = i + (e - i * W) - (k - 1);
    if (j < 0 || j >= N) {
        M1[e] = make_double2(0.0, 0.0);
        if (M2) M2[e] = make_double2(0.0, 0.0);
        return;
    }
    double a1 = 0.0, a2 = 0.0;
    int lo = max(max(i, j) - k + 2, 0), hi = min(min(i, j) + 1, n_iv - 1);
    for (int iv = lo; iv <= hi; ++iv) {
        double a = knots[k - 1 + iv], b = knots[k + iv];
        int si = i + 1 - iv, sj = j + 1 - iv;
        for (int P = 0; P < q; ++P) {
            size_t o = ((size_t)iv * q + P) * k;
            double x = tab_r[(size_t)iv * q + P], w = 0.5 * (b - a) * glw[P];
            double Bi = tab_B[o + si];
            if (gauge == 0) {
                a1 = a1 + w * x * Bi * tab_B[o + sj];
            } else {
                a1 = a1 + w * Bi * tab_D1[o + sj];
                a2 = a2 + w * Bi * tab_B[o + sj] / x;
            }
        }
    }
    if (gauge == 0) {
        M1[e] = make_double2(a1, 0.0);
    } else {  // multiply by -i
        M1[e] = make_double2(0.0, -a1);
        M2[e] = make_double2(0.0, -a2);
    }
}

}  // namespace

void launch_radial_dip(bs2e_handle *h, int gauge) {
    const Radial &g = h->g;
    int n = g.N * g.W;
    k_radial_dip<<<(n + 127) / 128, 128, 0, h->stream>>>(h->d_knots, h->d_glw, h->d_tab_r, h->d_tab_B,
                                                         h->d_tab_D1, g.k, g.q, g.N, g.n_iv, gauge,
                                                         h->d_dM1, h->d_dM2);
    h->launches++;
}

void launch_dip_count(bs2e_handle *h, const DipDev &D, int64_t *cnt) {
    DipArgs A{D.rows, D.n_rows, D.lmap_r, D.seg, D.seg + D.nseg, D.seg + 2 * D.nseg, h->g.N + 2,
              D.n_ch_r, D.n_ch_c, h->g.N, h->g.k, D.pairs, h->d_dM1, h->d_dM2, h->d_Sb};
    if (D.n_rows > 0) {
        k_dip_count<<<(unsigned)((D.n_rows + 127) / 128), 128, 0, h->stream>>>(A, cnt, D.stats);
        h->launches++;
    }
}

void launch_dip_fill(bs2e_handle *h, const DipDev &D, const int64_t *ptr, int64_t *idx,
                     double2 *dat) {
    DipArgs A{D.rows, D.n_rows, D.lmap_r, D.seg, D.seg + D.nseg, D.seg + 2 * D.nseg, h->g.N + 2,
              D.n_ch_r, D.n_ch_c, h->g.N, h->g.k, D.pairs, h->d_dM1, h->d_dM2, h->d_Sb};
    if (D.n_rows > 0) {
        const unsigned grid = (unsigned)((D.n_rows + 3) / 4);
        const int mode = h->s_real ? h->dip_kind : 0;
        if (mode == 1)
            k_dip_fill<1><<<grid, 128, 0, h->stream>>>(A, ptr, idx, dat);
        else if (mode == 2)
            k_dip_fill<2><<<grid, 128, 0, h->stream>>>(A, ptr, idx, dat);
        else
            k_dip_fill<0><<<grid, 128, 0, h->stream>>>(A, ptr, idx, dat);
        h->launches++;
    }
}

}  // namespace bs2e
