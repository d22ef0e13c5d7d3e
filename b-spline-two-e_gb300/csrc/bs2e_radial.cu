// bs2e_radial.cu -- radial stage on sm_103a: B-spline tabulation, per-interval
// moments, same-interval kink-split 2-D integrals, pair totals, the R^k store
// and the one-body matrices.
//
// Reference: src/mat_els/mat_els.f90:172-292 and 392-491 (Slater primitives),
// src/tools/sparse_array_tools.f90:452-493 (R^k accumulation),
// src/tools/bspline_tools.f90:151-224 (de Boor), mat_els.f90:47-118, 294-346
// (one-body S and H).
#include <cuda_runtime.h>

#include "bs2e_internal.h"

namespace bs2e {
namespace {

// De Boor value (or derivative) of the spline with unit coefficient at full
// index jsp (1-based) on interval iv1 (1-based), operation for operation as
// BVALUE_D with the interval hint (bspline_tools.f90:151-224).  Explicit
// round-to-nearest intrinsics keep the compiler from fusing multiply-adds, so
// the tables match an unfused CPU evaluation bit for bit.
__device__ double bval(const double *__restrict__ t, int k, double x, int ideriv, int iv1,
                       int jsp) {
    double aj[kMaxOrder + 2], dpv[kMaxOrder + 2], dmv[kMaxOrder + 2];
    int kmd = k - ideriv;
    if (kmd <= 0) return 0.0;
    int i = k - 1 + iv1;
#define T(idx) t[(idx)-1]
    for (int j = 1; j <= k; ++j) aj[j] = (i - k + j == jsp) ? 1.0 : 0.0;
    for (int j = 1; j <= ideriv; ++j) {
        int kmj = k - j;
        for (int jj = 1; jj <= kmj; ++jj) {
            int ihi = i + jj;
            double num = __dsub_rn(aj[jj + 1], aj[jj]);
            double den = __dsub_rn(T(ihi), T(ihi - kmj));
            aj[jj] = __dmul_rn(__ddiv_rn(num, den), (double)kmj);
        }
    }
    for (int j = 1; j <= kmd; ++j) {
        dpv[j] = __dsub_rn(T(i + j), x);
        dmv[j] = __dsub_rn(x, T(i + 1 - j));
    }
    for (int j = ideriv + 1; j <= k - 1; ++j) {
        int kmj = k - j;
        int ii = kmj;
        for (int jj = 1; jj <= kmj; ++jj) {
            double num = __dadd_rn(__dmul_rn(aj[jj + 1], dmv[ii]), __dmul_rn(aj[jj], dpv[jj]));
            aj[jj] = __ddiv_rn(num, __dadd_rn(dmv[ii], dpv[jj]));
            ii -= 1;
        }
    }
#undef T
    return aj[1];
}

// x^n by binary powering (the libgfortran real**integer scheme), n >= 0.
__device__ __forceinline__ double powi(double x, int n) {
    double p = 1.0;
    unsigned u = (unsigned)n;
    if (u == 0) return 1.0;
    for (;;) {
        if (u & 1u) p = __dmul_rn(p, x);
        u >>= 1;
        if (u)
            x = __dmul_rn(x, x);
        else
            break;
    }
    return p;
}

// ---------------------------------------------------------------------------
// K1: tabulation.  One CTA per breakpoint interval.
// ---------------------------------------------------------------------------
__global__ void k_tabulate(const double *__restrict__ knots, const double *__restrict__ glx,
                           int k, int q, double *__restrict__ tab_r, double *__restrict__ tab_B,
                           double *__restrict__ tab_D2, double *__restrict__ tab_D1,
                           double *__restrict__ tab_ri, double *__restrict__ tab_Bi) {
    const int iv = blockIdx.x;
    const int iv1 = iv + 1;
    const double lo = knots[k - 1 + iv], hi = knots[k + iv];
    const double sc = __dmul_rn(0.5, __dsub_rn(hi, lo));
    const double tr = __dmul_rn(0.5, __dadd_rn(hi, lo));
    for (int e = threadIdx.x; e < q * k; e += blockDim.x) {
        int P = e / k, s = e - P * k;
        double r = __dadd_rn(__dmul_rn(sc, glx[P]), tr);
        if (s == 0) tab_r[(size_t)iv * q + P] = r;
        tab_B[((size_t)iv * q + P) * k + s] = bval(knots, k, r, 0, iv1, iv1 + s);
        tab_D2[((size_t)iv * q + P) * k + s] = bval(knots, k, r, 2, iv1, iv1 + s);
        tab_D1[((size_t)iv * q + P) * k + s] = bval(knots, k, r, 1, iv1, iv1 + s);
    }
    for (int e = threadIdx.x; e < q * q * k; e += blockDim.x) {
        int s = e % k, PQ = e / k, Q = PQ % q, P = PQ / q;
        double r = __dadd_rn(__dmul_rn(sc, glx[P]), tr);
        double scj = __dmul_rn(0.5, __dsub_rn(r, lo));
        double trj = __dmul_rn(0.5, __dadd_rn(r, lo));
        double rj = __dadd_rn(__dmul_rn(scj, glx[Q]), trj);
        size_t o = ((size_t)iv * q + P) * q + Q;
        if (s == 0) tab_ri[o] = rj;
        tab_Bi[o * k + s] = bval(knots, k, rj, 0, iv1, iv1 + s);
    }
}

// ---------------------------------------------------------------------------
// K2: moments and same-interval integrals.  One CTA per (interval, multipole).
//   mom[iv][kk][0][s1][s2] = h sum_P w_P B_s1 B_s2 r_P^kk
//   mom[iv][kk][1][s1][s2] = h sum_P w_P B_s1 B_s2 / r_P^(kk+1)
//   dint[iv][kk][p][q]     = h sum_P (w_P B_i B_i' / r_P^(kk+1)) J_q(P),
//   J_q(P) = h_P sum_Q w_Q B_j(rho_PQ) B_j'(rho_PQ) rho_PQ^kk  on [t_iv, r_P]
// (compute_Slater_off_diag / compute_Slater_diag, mat_els.f90:392-491).
// ---------------------------------------------------------------------------
__global__ void k_moments(const double *__restrict__ knots, const double *__restrict__ glw, int k,
                          int q, int K1, const double *__restrict__ tab_r,
                          const double *__restrict__ tab_B, const double *__restrict__ tab_ri,
                          const double *__restrict__ tab_Bi, double *__restrict__ mom,
                          double *__restrict__ dint) {
    extern __shared__ double sm[];
    const int iv = blockIdx.x, kk = blockIdx.y;
    const int kq = k * q, k2 = k * k;
    double *sB = sm;              // [q][k]
    double *sR = sB + kq;         // [q]
    double *sBi = sR + q;         // [q][q][k]
    double *sRp = sBi + q * kq;   // [q][q] rho^kk
    double *sO = sRp + q * q;     // [k2][q]
    double *sJ = sO + k2 * q;     // [k2][q]
    double *sPk = sJ + k2 * q;    // [q] r^kk
    double *sPm = sPk + q;        // [q] r^(kk+1)
    double *sW = sPm + q;         // [q]
    for (int e = threadIdx.x; e < kq; e += blockDim.x) sB[e] = tab_B[(size_t)iv * kq + e];
    for (int e = threadIdx.x; e < q * kq; e += blockDim.x) sBi[e] = tab_Bi[(size_t)iv * q * kq + e];
    for (int e = threadIdx.x; e < q * q; e += blockDim.x)
        sRp[e] = powi(tab_ri[(size_t)iv * q * q + e], kk);
    for (int e = threadIdx.x; e < q; e += blockDim.x) {
        double r = tab_r[(size_t)iv * q + e];
        sR[e] = r;
        sPk[e] = powi(r, kk);
        sPm[e] = powi(r, kk + 1);
        sW[e] = glw[e];
    }
    __syncthreads();
    const double lo = knots[k - 1 + iv], hi = knots[k + iv];
    const double h = 0.5 * (hi - lo);
    const size_t mbase = ((size_t)iv * K1 + kk) * 2 * k2;
    for (int e = threadIdx.x; e < k2; e += blockDim.x) {
        int s1 = e / k, s2 = e - s1 * k;
        double a = 0.0, b = 0.0;
        for (int P = 0; P < q; ++P) {
            double wbb = sW[P] * sB[P * k + s1] * sB[P * k + s2];
            a = a + wbb * sPk[P];
            b = b + wbb / sPm[P];
        }
        mom[mbase + e] = h * a;
        mom[mbase + k2 + e] = h * b;
    }
    for (int e = threadIdx.x; e < k2 * q; e += blockDim.x) {
        int p = e / q, P = e - p * q;
        int si = p / k, sip = p - si * k;
        sO[e] = sW[P] * sB[P * k + si] * sB[P * k + sip] / sPm[P];
        int sj = si, sjp = sip;
        double hP = 0.5 * (sR[P] - lo);
        double acc = 0.0;
        for (int Q = 0; Q < q; ++Q) {
            const double *bq = sBi + (P * q + Q) * k;
            acc = acc + sW[Q] * bq[sj] * bq[sjp] * sRp[P * q + Q];
        }
        sJ[e] = hP * acc;
    }
    __syncthreads();
    const size_t dbase = ((size_t)iv * K1 + kk) * (size_t)k2 * k2;
    for (int e = threadIdx.x; e < k2 * k2; e += blockDim.x) {
        int p = e / k2, qq = e - p * k2;
        const double *o = sO + p * q;
        const double *jj = sJ + qq * q;
        double acc = 0.0;
        for (int P = 0; P < q; ++P) acc = fma(o[P], jj[P], acc);
        dint[dbase + e] = h * acc;
    }
}

// ---------------------------------------------------------------------------
// K3: pair totals tot[which][kk][a][dc] = sum over shared intervals of mom.
// ---------------------------------------------------------------------------
__global__ void k_totals(const double *__restrict__ mom, int k, int K1, int N, int n_iv,
                         double *__restrict__ tot) {
    const int W = 2 * k - 1;
    const int64_t total = (int64_t)2 * K1 * N * W;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        int dc = (int)(e % W);
        int64_t r = e / W;
        int a = (int)(r % N);
        r /= N;
        int kk = (int)(r % K1);
        int which = (int)(r / K1);
        int c = a + dc - (k - 1);
        double s = 0.0;
        if (c >= 0 && c < N) {
            int lo = max(max(a, c) - k + 2, 0), hi = min(min(a, c) + 1, n_iv - 1);
            for (int iv = lo; iv <= hi; ++iv) {
                int sa = a + 1 - iv, scc = c + 1 - iv;
                s += mom[(((size_t)iv * K1 + kk) * 2 + which) * k * k + sa * k + scc];
            }
        }
        tot[e] = s;
    }
}

// ---------------------------------------------------------------------------
// K4: R^k store.  One CTA per tile (a, b); element (kk, dc, dd) is
// R^k[a, b, c=a+dc-(k-1), d=b+dd-(k-1)] = sum over interval pairs (iv1 of the
// pair (a,c), iv2 of (b,d)) of
//   iv1 <  iv2 : m(ac,iv1) M(bd,iv2)   (r1 < r2)
//   iv1 >  iv2 : M(ac,iv1) m(bd,iv2)
//   iv1 == iv2 : D(iv; ac, bd) + D(iv; bd, ac)
// which is compute_R_K_map (sparse_array_tools.f90:472-488).  Pairs whose
// interval ranges do not overlap factor into one product of pair totals.
//
// MIXED stores each (tile, k) slice as FP32 pairs (hi, lo) of R 2^(kRkBias-e)
// with e = ilogb(max of the slice), and e in Rexp[tile][k]: hi + lo carries
// ~48 bits, and a slice may span up to ~2^180 before its smallest values lose
// precision (2^108 at the N=200, k=0..10 grid).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double rk_element(const double *__restrict__ mom,
                                            const double *__restrict__ dint,
                                            const double *__restrict__ tot, int k, int K1, int N,
                                            int n_iv, int a, int b, int kk, int dc, int dd) {
    const int W = 2 * k - 1, k2 = k * k;
    int c = a + dc - (k - 1), d = b + dd - (k - 1);
    if (c < 0 || c >= N || d < 0 || d >= N) return 0.0;
    int lop = max(max(a, c) - k + 2, 0), hip = min(min(a, c) + 1, n_iv - 1);
    int loq = max(max(b, d) - k + 2, 0), hiq = min(min(b, d) + 1, n_iv - 1);
    const double *mt = tot + (size_t)kk * N * W;
    const double *Mt = tot + ((size_t)K1 + kk) * N * W;
    if (hip < loq) return mt[a * W + dc] * Mt[b * W + dd];
    if (lop > hiq) return Mt[a * W + dc] * mt[b * W + dd];
    double v = 0.0;
    for (int iv1 = lop; iv1 <= hip; ++iv1) {
        int pa = (a + 1 - iv1) * k + (c + 1 - iv1);
        const double *m1 = mom + ((size_t)iv1 * K1 + kk) * 2 * k2;
        for (int iv2 = loq; iv2 <= hiq; ++iv2) {
            int pb = (b + 1 - iv2) * k + (d + 1 - iv2);
            const double *m2 = mom + ((size_t)iv2 * K1 + kk) * 2 * k2;
            if (iv1 < iv2) {
                v = fma(m1[pa], m2[k2 + pb], v);
            } else if (iv1 > iv2) {
                v = fma(m1[k2 + pa], m2[pb], v);
            } else {
                const double *D = dint + ((size_t)iv1 * K1 + kk) * (size_t)k2 * k2;
                v += D[(size_t)pa * k2 + pb] + D[(size_t)pb * k2 + pa];
            }
        }
    }
    return v;
}

__global__ void k_rk_store(const double *__restrict__ mom, const double *__restrict__ dint,
                          const double *__restrict__ tot, int k, int K1, int N, int n_iv,
                          int64_t tile, int k_first, int k_count, double *__restrict__ R) {
    const int W = 2 * k - 1, W2 = W * W;
    const int a = blockIdx.x / N, b = blockIdx.x - a * N;
    double *dst = R + (size_t)blockIdx.x * tile;
    const int nel = K1 * W2;
    for (int e = threadIdx.x; e < tile; e += blockDim.x) {
        if (e >= nel) {
            dst[e] = 0.0;
            continue;
        }
        int kk = e / W2, rem = e - kk * W2;
        if (kk < k_first || kk >= k_first + k_count) continue;
        int dc = rem / W, dd = rem - dc * W;
        dst[e] = rk_element(mom, dint, tot, k, K1, N, n_iv, a, b, kk, dc, dd);
    }
}

__global__ void k_rk_store_mixed(const double *__restrict__ mom, const double *__restrict__ dint,
                                const double *__restrict__ tot, int k, int K1, int N, int n_iv,
                                int64_t tile, int k_first, int k_count, float2 *__restrict__ Rf,
                                int *__restrict__ Rexp) {
    extern __shared__ double sv[];  // [K1][W][W] FP64 values of the tile
    __shared__ int sexp[kMaxK1];
    const int W = 2 * k - 1, W2 = W * W;
    const int a = blockIdx.x / N, b = blockIdx.x - a * N;
    const int nel = K1 * W2;
    for (int e = threadIdx.x; e < nel; e += blockDim.x) {
        int kk = e / W2, rem = e - kk * W2;
        if (kk < k_first || kk >= k_first + k_count) continue;
        int dc = rem / W, dd = rem - dc * W;
        sv[e] = rk_element(mom, dint, tot, k, K1, N, n_iv, a, b, kk, dc, dd);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    for (int kk = k_first + warp; kk < k_first + k_count; kk += nwarp) {
        double m = 0.0;
        for (int i = lane; i < W2; i += 32) m = fmax(m, sv[kk * W2 + i]);
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        int ex = (m > 0.0) ? ilogb(m) : 0;
        if (lane == 0) {
            sexp[kk] = ex;
            Rexp[(size_t)blockIdx.x * K1 + kk] = ex;
        }
    }
    __syncthreads();
    float2 *dst = Rf + (size_t)blockIdx.x * tile;
    for (int e = threadIdx.x; e < tile; e += blockDim.x) {
        if (e >= nel) {
            dst[e] = make_float2(0.f, 0.f);
            continue;
        }
        int kk = e / W2;
        if (kk < k_first || kk >= k_first + k_count) continue;
        double scale = __longlong_as_double((long long)(1023 + kRkBias - sexp[kk]) << 52);
        double x = sv[e] * scale;
        float hi = __double2float_rn(x);
        float lo = __double2float_rn(x - (double)hi);
        dst[e] = make_float2(hi, lo);
    }
}

__global__ void k_rk_gather(const double *__restrict__ R, const float2 *__restrict__ Rf,
                            const int *__restrict__ Rexp, int k, int K1, int N, int64_t tile,
                            int64_t n, const int64_t *__restrict__ keys, double *__restrict__ vals) {
    const int W = 2 * k - 1;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * K1;
         e += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = e / K1;
        int kk = (int)(e - i * K1);
        int64_t a = keys[4 * i] - 1, b = keys[4 * i + 1] - 1, c = keys[4 * i + 2] - 1,
                d = keys[4 * i + 3] - 1;
        double v = 0.0;
        if (a >= 0 && a < N && b >= 0 && b < N && c >= 0 && c < N && d >= 0 && d < N &&
            c - a < k && a - c < k && d - b < k && b - d < k) {
            int dc = (int)(c - a) + k - 1, dd = (int)(d - b) + k - 1;
            size_t t = (size_t)(a * N + b);
            size_t o = t * tile + ((size_t)kk * W + dc) * W + dd;
            if (R) {
                v = R[o];
            } else {
                float2 x = Rf[o];
                int ex = Rexp[t * K1 + kk];
                double scale = __longlong_as_double((long long)(1023 - kRkBias + ex) << 52);
                v = ((double)x.x + (double)x.y) * scale;
            }
        }
        vals[e] = v;
    }
}

// ---------------------------------------------------------------------------
// One-body matrices (setup_S, setup_H_one_particle: mat_els.f90:47-118,
// compute_H / compute_S :294-346) in banded form from the tabulated spline
// values and second derivatives at the interval GL points (the points gau_leg
// gives, quad_tools.f90:29-52).  One thread per (l, i, j) band entry, |i-j|<k:
//   H_l(i,j) = sum w (-1/2 B_i B_j'' + (l(l+1)/(2r^2) - Z/r + CAP(r)) B_i B_j)
// with CAP(r) = -i eta (r-r0)^order for r >= r0 (CAP_tools.f90:23-33).
// ---------------------------------------------------------------------------
__global__ void k_one_body(const double *__restrict__ knots, const double *__restrict__ glw,
                           const double *__restrict__ tab_r, const double *__restrict__ tab_B,
                           const double *__restrict__ tab_D2, int k, int q, int N, int n_iv,
                           int Z, int n_l, int cap_order, double cap_r0, double eta_re,
                           double eta_im, double2 *__restrict__ Sb, double2 *__restrict__ Hb) {
    const int W = 2 * k - 1;
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= (int64_t)n_l * N * W) return;
    const int l = (int)(e / ((int64_t)N * W));
    const int r = (int)(e - (int64_t)l * N * W);
    const int i = r / W, dx = r - i * W;  // 0-based basis index i, column j = i + dx - (k-1)
    const int j = i + dx - (k - 1);
    if (j < 0 || j >= N) {
        Hb[e] = make_double2(0.0, 0.0);
        if (l == 0) Sb[r] = make_double2(0.0, 0.0);
        return;
    }
    double s = 0.0, hre = 0.0, him = 0.0;
    const int lo = max(max(i, j) - k + 2, 0), hi = min(min(i, j) + 1, n_iv - 1);
    for (int iv = lo; iv <= hi; ++iv) {
        const double a = knots[k - 1 + iv], b = knots[k + iv];
        const int si = i + 1 - iv, sj = j + 1 - iv;
        for (int P = 0; P < q; ++P) {
            const size_t o = ((size_t)iv * q + P) * k;
            const double x = tab_r[(size_t)iv * q + P];
            const double w = 0.5 * (b - a) * glw[P];
            const double Bi = tab_B[o + si], Bj = tab_B[o + sj], DBj = tab_D2[o + sj];
            s = s + w * Bi * Bj;
            double cre = 0.0, cim = 0.0;
            if (x >= cap_r0) {
                double pw = powi(x - cap_r0, cap_order);
                cre = eta_im * pw;  // (0,-1) * eta * pw
                cim = -eta_re * pw;
            }
            const double V = 0.5 * (double)l * (double)(l + 1) / (x * x) - (double)Z / x;
            hre = hre + w * (-0.5 * Bi * DBj + (V + cre) * Bi * Bj);
            him = him + w * (cim * Bi * Bj);
        }
    }
    Hb[e] = make_double2(hre, him);
    if (l == 0) Sb[r] = make_double2(s, 0.0);
}

// Splits the complex FP64 bands into FP32 pairs (re hi, re lo, im hi, im lo)
// for the mixed assembly; flags any non-zero magnitude outside [2^-100, 2^100]
// so the host can keep FP64 one-body products instead.
__global__ void k_band_split(const double2 *__restrict__ src, int64_t n, float4 *__restrict__ dst,
                             int *__restrict__ flag) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x) {
        double2 v = src[e];
        float rh = __double2float_rn(v.x), ih = __double2float_rn(v.y);
        float rl = __double2float_rn(v.x - (double)rh), il = __double2float_rn(v.y - (double)ih);
        dst[e] = make_float4(rh, rl, ih, il);
        double ar = fabs(v.x), ai = fabs(v.y);
        const double lo = 7.888609052210118e-31, hi = 1.2676506002282294e+30;  // 2^-100, 2^100
        if ((ar != 0.0 && (ar < lo || ar > hi)) || (ai != 0.0 && (ai < lo || ai > hi)))
            atomicOr(flag, 1);
    }
}

}  // namespace

static inline unsigned grid_for(int64_t n, int threads) {
    int64_t g = (n + threads - 1) / threads;
    if (g > (int64_t)152 * 64) g = (int64_t)152 * 64;
    if (g < 1) g = 1;
    return (unsigned)g;
}

void launch_tabulate(bs2e_handle *h) {
    const Radial &g = h->g;
    k_tabulate<<<g.n_iv, 128, 0, h->stream>>>(h->d_knots, h->d_glx, g.k, g.q, h->d_tab_r,
                                               h->d_tab_B, h->d_tab_D2, h->d_tab_D1, h->d_tab_ri,
                                               h->d_tab_Bi);
    h->launches++;
}

size_t moments_smem(const Radial &g) {
    int k = g.k, q = g.q, kq = k * q, k2 = k * k;
    return sizeof(double) * (size_t)(kq + q + q * kq + q * q + 2 * k2 * q + 3 * q);
}

void launch_moments(bs2e_handle *h) {
    const Radial &g = h->g;
    size_t smem = moments_smem(g);
    cudaFuncSetAttribute(k_moments, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid(g.n_iv, g.K1);
    k_moments<<<grid, 256, smem, h->stream>>>(h->d_knots, h->d_glw, g.k, g.q, g.K1, h->d_tab_r,
                                              h->d_tab_B, h->d_tab_ri, h->d_tab_Bi, h->d_mom,
                                              h->d_dint);
    h->launches++;
}

void launch_totals(bs2e_handle *h) {
    const Radial &g = h->g;
    int64_t n = (int64_t)2 * g.K1 * g.N * g.W;
    k_totals<<<grid_for(n, 256), 256, 0, h->stream>>>(h->d_mom, g.k, g.K1, g.N, g.n_iv, h->d_tot);
    h->launches++;
}

void launch_rk_fill(bs2e_handle *h, int k_first, int k_count) {
    const Radial &g = h->g;
    unsigned tiles = (unsigned)((int64_t)g.N * g.N);
    if (h->precision == BS2E_PREC_MIXED) {
        size_t smem = (size_t)g.K1 * g.W * g.W * sizeof(double);
        cudaFuncSetAttribute(k_rk_store_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_rk_store_mixed<<<tiles, 256, smem, h->stream>>>(h->d_mom, h->d_dint, h->d_tot, g.k, g.K1,
                                                         g.N, g.n_iv, g.tile, k_first, k_count,
                                                         h->d_Rf, h->d_Rexp);
    } else {
        k_rk_store<<<tiles, 256, 0, h->stream>>>(h->d_mom, h->d_dint, h->d_tot, g.k, g.K1, g.N,
                                                g.n_iv, g.tile, k_first, k_count, h->d_R);
    }
    h->launches++;
}

void launch_rk_gather(bs2e_handle *h, int64_t n, const int64_t *d_keys, double *d_vals) {
    const Radial &g = h->g;
    k_rk_gather<<<grid_for(n * g.K1, 256), 256, 0, h->stream>>>(
        h->d_R, h->d_Rf, h->d_Rexp, g.k, g.K1, g.N, g.tile, n, d_keys, d_vals);
    h->launches++;
}

void launch_band_split(bs2e_handle *h) {
    const Radial &g = h->g;
    int64_t nh = h->n_l * g.N * g.W, ns = (int64_t)g.N * g.W;
    cudaMemsetAsync(h->d_flag, 0, sizeof(int), h->stream);
    k_band_split<<<grid_for(nh, 256), 256, 0, h->stream>>>(h->d_Hb, nh, h->d_Hbf, h->d_flag);
    k_band_split<<<grid_for(ns, 256), 256, 0, h->stream>>>(h->d_Sb, ns, h->d_Sbf, h->d_flag);
    h->launches += 2;
}

void launch_one_body(bs2e_handle *h, int64_t Z, int64_t n_l, int64_t cap_order, double cap_r0,
                     double eta_re, double eta_im) {
    const Radial &g = h->g;
    int64_t n = n_l * g.N * g.W;
    k_one_body<<<(unsigned)((n + 127) / 128), 128, 0, h->stream>>>(
        h->d_knots, h->d_glw, h->d_tab_r, h->d_tab_B, h->d_tab_D2, g.k, g.q, g.N, g.n_iv, (int)Z,
        (int)n_l, (int)cap_order, cap_r0, eta_re, eta_im, h->d_Sb, h->d_Hb);
    h->launches++;
}

}  // namespace bs2e
