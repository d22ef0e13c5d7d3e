// bs2e_radial.cu -- radial stage on sm_103a: B-spline tabulation, per-interval
// moments, same-interval kink-split 2-D integrals, pair totals, the R^k store
// and the one-body matrices.
//
// Reference: src/mat_els/mat_els.f90:172-292 and 392-491 (Slater primitives),
// src/tools/sparse_array_tools.f90:452-493 (R^k accumulation),
// src/tools/bspline_tools.f90:151-224 (de Boor), mat_els.f90:47-118, 294-346
// (one-body S and H).
#include <cuda_runtime.h>

#include <algorithm>

#include "bs2e_dmul.h"
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
// K1: tabulation.  Part `part` of `nparts` CTAs of a breakpoint interval (the
// batched stage runs a whole interval per work item: part 0 of 1).
// ---------------------------------------------------------------------------
__device__ void tabulate_iv(const RadialDev &P, int iv, int part = 0, int nparts = 1) {
    const int k = P.k, q = P.q;
    const double *__restrict__ knots = P.knots;
    const double *__restrict__ glx = P.glx;
    const int iv1 = iv + 1;
    const double lo = knots[k - 1 + iv], hi = knots[k + iv];
    const double sc = __dmul_rn(0.5, __dsub_rn(hi, lo));
    const double tr = __dmul_rn(0.5, __dadd_rn(hi, lo));
    const int e0 = part * blockDim.x + threadIdx.x, es = nparts * blockDim.x;
    for (int e = e0; e < q * k; e += es) {
        int Pp = e / k, s = e - Pp * k;
        double r = __dadd_rn(__dmul_rn(sc, glx[Pp]), tr);
        if (s == 0) P.tab_r[(size_t)iv * q + Pp] = r;
        P.tab_B[((size_t)iv * q + Pp) * k + s] = bval(knots, k, r, 0, iv1, iv1 + s);
        P.tab_D2[((size_t)iv * q + Pp) * k + s] = bval(knots, k, r, 2, iv1, iv1 + s);
        P.tab_D1[((size_t)iv * q + Pp) * k + s] = bval(knots, k, r, 1, iv1, iv1 + s);
    }
    for (int e = e0; e < q * q * k; e += es) {
        int s = e % k, PQ = e / k, Q = PQ % q, Pp = PQ / q;
        double r = __dadd_rn(__dmul_rn(sc, glx[Pp]), tr);
        double scj = __dmul_rn(0.5, __dsub_rn(r, lo));
        double trj = __dmul_rn(0.5, __dadd_rn(r, lo));
        double rj = __dadd_rn(__dmul_rn(scj, glx[Q]), trj);
        size_t o = ((size_t)iv * q + Pp) * q + Q;
        if (s == 0) P.tab_ri[o] = rj;
        P.tab_Bi[o * k + s] = bval(knots, k, rj, 0, iv1, iv1 + s);
    }
}

__global__ void k_tabulate(RadialDev P) { tabulate_iv(P, blockIdx.x, blockIdx.y, gridDim.y); }

// ---------------------------------------------------------------------------
// K2: moments and same-interval integrals.  One CTA per (interval, multipole).
//   mom[iv][kk][0][s1][s2] = h sum_P w_P B_s1 B_s2 r_P^kk
//   mom[iv][kk][1][s1][s2] = h sum_P w_P B_s1 B_s2 / r_P^(kk+1)
//   dint[iv][kk][p][q]     = h sum_P (w_P B_i B_i' / r_P^(kk+1)) J_q(P),
//   J_q(P) = h_P sum_Q w_Q B_j(rho_PQ) B_j'(rho_PQ) rho_PQ^kk  on [t_iv, r_P]
// (compute_Slater_off_diag / compute_Slater_diag, mat_els.f90:392-491).
// ---------------------------------------------------------------------------
__device__ void moments_item(const RadialDev &Pd, int iv, int kk, double *sm) {
    const int k = Pd.k, q = Pd.q, K1 = Pd.K1;
    const double *__restrict__ knots = Pd.knots;
    const double *__restrict__ glw = Pd.glw;
    const double *__restrict__ tab_r = Pd.tab_r;
    const double *__restrict__ tab_B = Pd.tab_B;
    const double *__restrict__ tab_ri = Pd.tab_ri;
    const double *__restrict__ tab_Bi = Pd.tab_Bi;
    double *__restrict__ mom = Pd.mom;
    double *__restrict__ dint = Pd.dint;
    const int kq = k * q, k2 = k * k;
    double *sB = sm;              // [q][k]
    double *sR = sB + kq;         // [q]
    double *sBi = sR + q;         // [q][q][k]
    double *sRp = sBi + q * kq;   // [q][q] rho^kk
    double *sO = sRp + q * q;     // [k2][q]
    double *sJ = sO + k2 * q;     // [k2][q]
    double *sPk = sJ + k2 * q;    // [q] r^kk
    double *sPm = sPk + q;        // [q] 1 / r^(kk+1)
    double *sW = sPm + q;         // [q]
    for (int e = threadIdx.x; e < kq; e += blockDim.x) sB[e] = tab_B[(size_t)iv * kq + e];
    for (int e = threadIdx.x; e < q * kq; e += blockDim.x) sBi[e] = tab_Bi[(size_t)iv * q * kq + e];
    for (int e = threadIdx.x; e < q * q; e += blockDim.x)
        sRp[e] = powi(tab_ri[(size_t)iv * q * q + e], kk);
    for (int e = threadIdx.x; e < q; e += blockDim.x) {
        double r = tab_r[(size_t)iv * q + e];
        sR[e] = r;
        sPk[e] = powi(r, kk);
        // one division per point; the sums below multiply by it (within a
        // rounding of dividing each term, far inside the parity bars)
        sPm[e] = 1.0 / powi(r, kk + 1);
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
            b = b + wbb * sPm[P];
        }
        mom[mbase + e] = h * a;
        mom[mbase + k2 + e] = h * b;
    }
    for (int e = threadIdx.x; e < k2 * q; e += blockDim.x) {
        int p = e / q, P = e - p * q;
        int si = p / k, sip = p - si * k;
        sO[e] = sW[P] * sB[P * k + si] * sB[P * k + sip] * sPm[P];
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
    // (p, qq) of e = p * k2 + qq walked incrementally (no division per element)
    const int step_p = blockDim.x / k2, step_q = blockDim.x - step_p * k2;
    int p = threadIdx.x / k2, qq = threadIdx.x - p * k2;
    for (int e = threadIdx.x; e < k2 * k2; e += blockDim.x) {
        const double *o = sO + p * q;
        const double *jj = sJ + qq * q;
        double acc = 0.0;
        for (int P = 0; P < q; ++P) acc = fma(o[P], jj[P], acc);
        dint[dbase + e] = h * acc;
        p += step_p;
        qq += step_q;
        if (qq >= k2) {
            qq -= k2;
            ++p;
        }
    }
    // the symmetric sums D(p, q) + D(q, p) the R^k store adds per shared
    // interval, formed once here (the same additions, so the store is the
    // same bit for bit); the barrier makes the CTA's D writes visible
    __syncthreads();
    double *__restrict__ dsym = Pd.dsym;
    p = threadIdx.x / k2;
    qq = threadIdx.x - p * k2;
    for (int e = threadIdx.x; e < k2 * k2; e += blockDim.x) {
        dsym[dbase + e] = dint[dbase + e] + dint[dbase + (size_t)qq * k2 + p];
        p += step_p;
        qq += step_q;
        if (qq >= k2) {
            qq -= k2;
            ++p;
        }
    }
}

__global__ void k_moments(RadialDev P) {
    extern __shared__ double sm[];
    moments_item(P, blockIdx.x, blockIdx.y, sm);
}

// ---------------------------------------------------------------------------
// K3: pair totals tot[which][kk][a][dc] = sum over shared intervals of mom.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void totals_elem(const RadialDev &P, int64_t e) {
    const int k = P.k, K1 = P.K1, N = P.N, n_iv = P.n_iv, W = 2 * k - 1;
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
            s += P.mom[(((size_t)iv * K1 + kk) * 2 + which) * k * k + sa * k + scc];
        }
    }
    P.tot[e] = s;
}

__device__ __forceinline__ int64_t totals_count(const RadialDev &P) {
    return (int64_t)2 * P.K1 * P.N * (2 * P.k - 1);
}

__global__ void k_totals(RadialDev P) {
    const int64_t total = totals_count(P);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x)
        totals_elem(P, e);
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
// ~48 bits, and a slice may span up to ~2^214 before its smallest values lose
// precision (2^108 at the N=200, k=0..10 grid; about 2^200 at k=20 on the
// N=800, r_max=800 grid).
// ---------------------------------------------------------------------------

// Near-field tiles (|a - b| < k, where the interval ranges of an (a, c) pair
// and a (b, d) pair can meet).  With iv2_j = b - k + 2 + j (j < k) the
// intervals a (b, d) pair can use, the two triangles of the interval-pair
// sum factor through prefix sums over the (a, c) intervals,
//   Pm[j] = sum_{iv1 < iv2_j} m(ac, iv1),    SM[j] = sum_{iv1 > iv2_j} M(ac, iv1),
//   R = sum_j ( M(bd, iv2_j) Pm[j] + m(bd, iv2_j) SM[j] )
//       + sum_{shared iv} D(iv; ac, bd) + D(iv; bd, ac),
// 2k FMAs per element instead of up to k^2 products.  Both sums add
// positive moments (B-splines are non-negative), so the regrouping keeps full
// accuracy.  Staged per multipole in s[4][k][W]: Pm, SM over dc; m, M over dd;
// multipoles [g0, g0 + gn) at once, multipole g0 + i at s + i * 4kW.  One
// thread per (multipole, dc) builds Pm[.][dc] as a running sum over ascending
// iv1 (each j adds the intervals iv2_j newly passes) and another SM[.][dc]
// from the top down, so the (a, c) moments are read and added once each.
__device__ void rk_near_stage(const RadialDev &P, int a, int b, int g0, int gn, double *sg) {
    const int k = P.k, K1 = P.K1, N = P.N, n_iv = P.n_iv, W = 2 * k - 1, k2 = k * k;
    const int base2 = b - k + 2, per = 4 * W * k;
    const double *__restrict__ mom = P.mom;
    // (a, c) part: prefix (x even) and suffix (x odd) walkers
    for (int x = threadIdx.x; x < gn * 2 * W; x += blockDim.x) {
        const int gi = x / (2 * W), r = x - gi * 2 * W, off = r >> 1, kk = g0 + gi;
        const bool suf = r & 1;
        double *s = sg + (size_t)gi * per + (suf ? k * W : 0) + off;  // s[j * W]
        const int c = a + off - (k - 1);
        int lop = 0, hip = -1;
        if (c >= 0 && c < N) {
            lop = max(max(a, c) - k + 2, 0);
            hip = min(min(a, c) + 1, n_iv - 1);
        }
        const double *mk = mom + (size_t)kk * 2 * k2 + (suf ? k2 : 0) + (a + 1) * k + (c + 1);
        // moment of interval iv: mk[iv * (K1 2 k^2) - iv * (k + 1)]
        const size_t ivs = (size_t)K1 * 2 * k2 - (k + 1);
        double v = 0.0;
        if (!suf) {
            int iv1 = lop;
            for (int j = 0; j < k; ++j) {
                for (const int lim = min(hip, base2 + j - 1); iv1 <= lim; ++iv1) v += mk[iv1 * ivs];
                s[j * W] = v;  // Pm: sum over iv1 < iv2_j
            }
        } else {
            int iv1 = hip;
            for (int j = k - 1; j >= 0; --j) {
                for (const int lim = max(lop, base2 + j + 1); iv1 >= lim; --iv1) v += mk[iv1 * ivs];
                s[j * W] = v;  // SM: sum over iv1 > iv2_j
            }
        }
    }
    // (b, d) part: the moments of the (b, d) pair on iv2_j
    for (int xg = threadIdx.x; xg < gn * W * k; xg += blockDim.x) {
        const int gi = xg / (W * k), y = xg - gi * W * k, kk = g0 + gi;
        double *s = sg + (size_t)gi * per;
        const int off = y / k, j = y - off * k;
        const int iv2 = base2 + j;
        double v0 = 0.0, v1 = 0.0;
        const int d = b + off - (k - 1);
        if (d >= 0 && d < N) {
            const int loq = max(max(b, d) - k + 2, 0), hiq = min(min(b, d) + 1, n_iv - 1);
            if (iv2 >= loq && iv2 <= hiq) {
                const double *m2 = mom + ((size_t)iv2 * K1 + kk) * 2 * k2;
                const int pb = (b + 1 - iv2) * k + (d + 1 - iv2);
                v0 = m2[pb];
                v1 = m2[k2 + pb];
            }
        }
        s[(2 * k + j) * W + off] = v0;  // m(bd)
        s[(3 * k + j) * W + off] = v1;  // M(bd)
    }
}

__device__ __forceinline__ double rk_near_element(const RadialDev &P, const double *s, int a,
                                                  int b, int kk, int dc, int dd) {
    const int k = P.k, K1 = P.K1, N = P.N, n_iv = P.n_iv, W = 2 * k - 1, k2 = k * k;
    const int c = a + dc - (k - 1), d = b + dd - (k - 1);
    if (c < 0 || c >= N || d < 0 || d >= N) return 0.0;
    double v = 0.0;
    // m(bd) and M(bd) vanish off the (b, d) pair's intervals, iv2_j in
    // [max(b, d) - k + 2, min(b, d) + 1]: the terms skipped there are exact
    // zeros, so the sum is the same bit for bit
    const int jlo = max(0, d - b), jhi = k - 1 + min(0, d - b);
    for (int j = jlo; j <= jhi; ++j) {
        v = fma(s[(3 * k + j) * W + dd], s[j * W + dc], v);
        v = fma(s[(2 * k + j) * W + dd], s[(k + j) * W + dc], v);
    }
    const int lo = max(max(max(a, c), max(b, d)) - k + 2, 0);
    const int hi = min(min(min(a, c), min(b, d)) + 1, n_iv - 1);
    for (int iv = lo; iv <= hi; ++iv) {
        const int pa = (a + 1 - iv) * k + (c + 1 - iv), pb = (b + 1 - iv) * k + (d + 1 - iv);
        // D(iv; ac, bd) + D(iv; bd, ac), summed once by the moments stage
        v += P.dsym[((size_t)iv * K1 + kk) * (size_t)k2 * k2 + (size_t)pa * k2 + pb];
    }
    return v;
}

// Multipoles staged together in a near-field tile: as many stages s[4][k][W]
// as fit in about 20 KB, so a tile takes few barrier pairs and every thread
// has elements to compute.
__host__ __device__ __forceinline__ int rk_near_group(int k, int K1) {
    const int one = 4 * k * (2 * k - 1), g = 2560 / one;
    return g < 1 ? 1 : (g > K1 ? K1 : g);
}

// Scratch doubles of a tile: the near-field stages of a group or the
// far-field pair totals [2][K1][W].
__host__ __device__ __forceinline__ size_t rk_scratch(int k, int K1) {
    const size_t W = 2 * k - 1, near = 4 * (size_t)k * W * rk_near_group(k, K1);
    const size_t far = 2 * (size_t)K1 * W;
    return near > far ? near : far;
}

// Values of multipoles [k_first, k_first + k_count) of tile t = a * N + b:
// out[kk * W^2 + dc * W + dd] (block-wide; s: rk_scratch doubles).  Each
// thread takes the elements blockDim apart from its own and walks them with an
// incremental (kk, dc, dd), so no element pays an integer division.
template <int INTQ>
__device__ void rk_tile_values(const RadialDev &P, int64_t t, int k_first, int k_count,
                               double *out, double *s) {
    const int k = P.k, K1 = P.K1, N = P.N, W = 2 * k - 1, W2 = W * W;
    const int a = (int)(t / N), b = (int)(t - (int64_t)a * N);
    // a thread's elements lie blockDim apart: that stride as (multipoles, dc, dd)
    const int S = blockDim.x, sk = S / W2, sdc = (S - sk * W2) / W;
    const int sdd = S - sk * W2 - sdc * W;
    if (abs(a - b) >= k) {
        // far field everywhere: the (a, c) intervals lie all below the (b, d)
        // ones when a < b, all above when a > b, so R^k is the product of the
        // pair totals, X = m_k(ac) and Y = M_k(bd), or X = M_k(ac) and
        // Y = m_k(bd) (sparse_array_tools.f90:452-493 sums the same interval
        // products).  The totals are 0 where c or d falls off the grid, so
        // those elements come out as +0.
        const size_t NW = (size_t)N * W, lower = a < b ? 0 : (size_t)K1 * NW;
        const size_t upper = a < b ? (size_t)K1 * NW : 0;
        double *sx = s, *sy = s + (size_t)K1 * W;  // [K1][W] each
        for (int i = threadIdx.x; i < k_count * W; i += blockDim.x) {
            const int kq = i / W, off = i - kq * W, kk = k_first + kq;
            sx[kk * W + off] = P.tot[lower + kk * NW + (size_t)a * W + off];
            sy[kk * W + off] = P.tot[upper + kk * NW + (size_t)b * W + off];
        }
        __syncthreads();
        // every thread walks elements e = kk W^2 + dc W + dd, blockDim apart,
        // with an incremental (kk, dc, dd); one product per stored element,
        // INTQ of every four warps on the integer pipes (bit for bit the FP64
        // multiply; bs2e_dmul.h says why) and the others on the FP64 pipe, so
        // the two pipes share the products
        const int e1 = (k_first + k_count) * W2;
        int e = k_first * W2 + threadIdx.x;
        int kk = e / W2, dc = (e - kk * W2) / W, dd = e - kk * W2 - dc * W;
        if (((threadIdx.x >> 5) & 3) < INTQ) {
            for (; e < e1; e += S) {
                out[e] = dmul_int(sx[kk * W + dc], sy[kk * W + dd]);
                kk += sk; dc += sdc; dd += sdd;
                if (dd >= W) { dd -= W; ++dc; }
                if (dc >= W) { dc -= W; ++kk; }
            }
        } else {
            for (; e < e1; e += S) {
                out[e] = sx[kk * W + dc] * sy[kk * W + dd];
                kk += sk; dc += sdc; dd += sdd;
                if (dd >= W) { dd -= W; ++dc; }
                if (dc >= W) { dc -= W; ++kk; }
            }
        }
        return;
    }
    const int G = rk_near_group(k, K1), per = 4 * k * W;
    for (int g0 = k_first; g0 < k_first + k_count; g0 += G) {
        const int gn = min(G, k_first + k_count - g0);
        __syncthreads();  // the previous group's elements are done with s
        rk_near_stage(P, a, b, g0, gn, s);
        __syncthreads();
        // the group's elements taken in the order (dd, dc, multipole), so the
        // lanes of a warp share dd and span few dc: both loops of
        // rk_near_element run over intervals of the (b, d) pair (the second
        // also of the (a, c) pair), and with d common and c close their trip
        // counts agree across the warp instead of every lane waiting for the
        // longest (the stores go out W^2 apart, on these few tiles only)
        const int GW = gn * W, tdd = S / GW, tdc = (S - tdd * GW) / gn;
        const int tgi = S - tdd * GW - tdc * gn;
        int e = threadIdx.x, dd = e / GW, dc = (e - dd * GW) / gn, gi = e - dd * GW - dc * gn;
        for (; e < gn * W2; e += S) {
            out[(size_t)(g0 + gi) * W2 + dc * W + dd] =
                rk_near_element(P, s + (size_t)gi * per, a, b, g0 + gi, dc, dd);
            dd += tdd; dc += tdc; gi += tgi;
            if (gi >= gn) { gi -= gn; ++dc; }
            if (dc >= W) { dc -= W; ++dd; }
        }
    }
}

// Tile t = a * N + b of the FP64 store (block-wide).
template <int INTQ>
__device__ void rk_tile_fp64(const RadialDev &P, int64_t t, int k_first, int k_count, double *s) {
    const int k = P.k, K1 = P.K1, W = 2 * k - 1;
    double *dst = P.R + (size_t)t * P.tile;
    const int nel = K1 * W * W;
    for (int e = nel + threadIdx.x; e < P.tile; e += blockDim.x) dst[e] = 0.0;
    rk_tile_values<INTQ>(P, t, k_first, k_count, dst, s);
}

// Tile t of the mixed store (block-wide); sv holds K1 W^2 doubles.
template <int INTQ>
__device__ void rk_tile_mixed(const RadialDev &P, int64_t t, int k_first, int k_count,
                              double *sv, int *sexp, double *s) {
    const int k = P.k, K1 = P.K1, W = 2 * k - 1, W2 = W * W;
    const int nel = K1 * W2;
    rk_tile_values<INTQ>(P, t, k_first, k_count, sv, s);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    for (int kk = k_first + warp; kk < k_first + k_count; kk += nwarp) {
        // the slice maximum through the bit patterns (non-negative doubles
        // order as unsigned integers), off the FP64 pipe
        unsigned long long m = 0ull;
        for (int i = lane; i < W2; i += 32)
            m = max(m, (unsigned long long)__double_as_longlong(sv[kk * W2 + i]));
        for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
        int ex = m ? (int)(m >> 52) - 1023 : 0;  // ilogb of the (normal) maximum
        if (lane == 0) {
            sexp[kk] = ex;
            P.Rexp[(size_t)t * K1 + kk] = ex;
        }
    }
    __syncthreads();
    float2 *dst = P.Rf + (size_t)t * P.tile;
    for (int e = nel + threadIdx.x; e < P.tile; e += blockDim.x) dst[e] = make_float2(0.f, 0.f);
    for (int kk = k_first; kk < k_first + k_count; ++kk) {
        const int s = kRkBias - sexp[kk];
        for (int r = threadIdx.x; r < W2; r += blockDim.x) {
            const int e = kk * W2 + r;
            // (hi, lo) of sv[e] 2^s as the FP64 conversions give them, formed on
            // the integer pipes (bs2e_dmul.h)
            float hi, lo;
            split_scaled(sv[e], s, hi, lo);
            dst[e] = make_float2(hi, lo);
        }
    }
}

// Quarters of the warps whose far-field products run on the integer pipes.
// Measured (R^k store, FP64, ms) at order 9 N=800 k<=20 / order 9 N=200 /
// order 7 N=200 and the 64-problem ragged batch: 0/4 -> 10.38 / 1.24 / 0.338
// / 91.3; 1/4 -> 9.66 / 1.19 / 0.343 / 97.8; 2/4 -> 10.09 / 1.20 / 0.361 /
// 98.7; 3/4 -> 12.63 / 1.26 / 0.398 / 103.6.  The batched kernel, capped at
// 64 registers, keeps every product on the FP64 pipe.
constexpr int kRkIntQuartersSingle = 1;
constexpr int kRkIntQuartersBatch = 0;

__global__ void k_rk_store(RadialDev P, int k_first, int k_count) {
    extern __shared__ double scr[];  // rk_scratch(k, K1) doubles
    rk_tile_fp64<kRkIntQuartersSingle>(P, blockIdx.x, k_first, k_count, scr);
}

__global__ void k_rk_store_mixed(RadialDev P, int k_first, int k_count) {
    extern __shared__ double sv[];  // [K1][W][W] FP64 values of the tile, then the scratch
    __shared__ int sexp[kMaxK1];
    rk_tile_mixed<kRkIntQuartersSingle>(P, blockIdx.x, k_first, k_count, sv, sexp,
                  sv + (size_t)P.K1 * (2 * P.k - 1) * (2 * P.k - 1));
}

// ---------------------------------------------------------------------------
// Batched radial stage: one persistent kernel per stage runs that stage of
// every problem of a batch.  Items [off[p], off[p+1]) belong to problem p
// (0: intervals, 1: (interval, multipole), 2: chunks of blockDim totals,
// 3: R^k tiles of the FP64 problems, 4: R^k tiles of the mixed ones); a CTA
// takes `chunk` consecutive items per atomicAdd on the stage's counter until
// the queue is empty.  No CTA waits on another.  The R^k stages are separate
// kernels per store type and capped at 64 registers (256 threads, 4 CTAs per
// SM), the occupancy of the single-problem k_rk_store.
// ---------------------------------------------------------------------------
struct BatchStage {
    const RadialDev *probs;
    const int64_t *off;  // [n + 1]
    int n, chunk;
    int persistent;  // 1: CTAs drain the queue; 0: CTA x takes items [x chunk, (x + 1) chunk)
    unsigned long long *counter;
};

__device__ __forceinline__ int find_problem(const int64_t *off, int n, int64_t it) {
    int lo = 0, hi = n - 1;  // largest p with off[p] <= it
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= it)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

template <int STAGE>
__device__ __forceinline__ void batch_body(const BatchStage &B) {
    extern __shared__ double sm[];
    __shared__ int sexp[kMaxK1];
    __shared__ unsigned long long s_it;
    const int64_t total = B.off[B.n];
    for (int pass = 0;; ++pass) {
        if (B.persistent) {
            if (threadIdx.x == 0) s_it = atomicAdd(B.counter, (unsigned long long)B.chunk);
        } else if (threadIdx.x == 0) {
            s_it = pass == 0 ? (unsigned long long)blockIdx.x * B.chunk : (unsigned long long)total;
        }
        __syncthreads();
        const int64_t it0 = (int64_t)s_it;
        __syncthreads();
        if (it0 >= total) break;
        const int64_t it1 = min(it0 + (int64_t)B.chunk, total);
        for (int64_t it = it0; it < it1; ++it) {
            const int p = find_problem(B.off, B.n, it);
            const RadialDev P = B.probs[p];
            const int64_t li = it - B.off[p];
            if (STAGE == 0) {
                tabulate_iv(P, (int)li);
            } else if (STAGE == 1) {
                moments_item(P, (int)(li / P.K1), (int)(li % P.K1), sm);
                __syncthreads();  // shared arrays are rewritten by the next item
            } else if (STAGE == 2) {
                const int64_t e = li * blockDim.x + threadIdx.x;
                if (e < totals_count(P)) totals_elem(P, e);
            } else if (STAGE == 3) {
                rk_tile_fp64<kRkIntQuartersBatch>(P, li, 0, P.K1, sm);
                __syncthreads();
            } else {
                rk_tile_mixed<kRkIntQuartersBatch>(P, li, 0, P.K1, sm, sexp,
                              sm + (size_t)P.K1 * (2 * P.k - 1) * (2 * P.k - 1));
                __syncthreads();
            }
        }
    }
}

template <int STAGE>
__global__ void k_radial_batch(BatchStage B) {
    batch_body<STAGE>(B);
}

template <int STAGE>
__global__ void __launch_bounds__(256, 4) k_radial_batch_rk(BatchStage B) {
    batch_body<STAGE>(B);
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

// Multipole kk of the whole store as doubles, out[a][b][c-a+k-1][d-b+k-1]
// (0-based a, b; zero where c or d falls outside the basis).
__global__ void k_rk_slice(const double *__restrict__ R, const float2 *__restrict__ Rf,
                           const int *__restrict__ Rexp, int kk, int k, int K1, int N,
                           int64_t tile, double *__restrict__ out) {
    const int W = 2 * k - 1;
    const int64_t n = (int64_t)N * N * W * W;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = e / (W * W);
        const int r = (int)(e - t * W * W), dc = r / W, dd = r - dc * W;
        const int a = (int)(t / N), b = (int)(t - (int64_t)a * N);
        const int c = a + dc - (k - 1), d = b + dd - (k - 1);
        double v = 0.0;
        if (c >= 0 && c < N && d >= 0 && d < N) {
            const size_t o = (size_t)t * tile + ((size_t)kk * W + dc) * W + dd;
            if (R) {
                v = R[o];
            } else {
                const float2 x = Rf[o];
                const int ex = Rexp[(size_t)t * K1 + kk];
                v = ((double)x.x + (double)x.y) *
                    __longlong_as_double((long long)(1023 - kRkBias + ex) << 52);
            }
        }
        out[e] = v;
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
    // one warp per band entry: the lanes take the (interval, point) terms of
    // its quadrature and a shuffle reduction sums them
    const int W = 2 * k - 1;
    const int64_t e = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (e >= (int64_t)n_l * N * W) return;  // whole warp
    const int l = (int)(e / ((int64_t)N * W));
    const int r = (int)(e - (int64_t)l * N * W);
    const int i = r / W, dx = r - i * W;  // 0-based basis index i, column j = i + dx - (k-1)
    const int j = i + dx - (k - 1);
    if (j < 0 || j >= N) {
        if (lane == 0) {
            Hb[e] = make_double2(0.0, 0.0);
            if (l == 0) Sb[r] = make_double2(0.0, 0.0);
        }
        return;
    }
    double s = 0.0, hre = 0.0, him = 0.0;
    const int lo = max(max(i, j) - k + 2, 0), hi = min(min(i, j) + 1, n_iv - 1);
    for (int t = lane; t < (hi - lo + 1) * q; t += 32) {
        const int iv = lo + t / q, P = t - (iv - lo) * q;
        const double a = knots[k - 1 + iv], b = knots[k + iv];
        const int si = i + 1 - iv, sj = j + 1 - iv;
        {
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
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        hre += __shfl_xor_sync(0xffffffffu, hre, o);
        him += __shfl_xor_sync(0xffffffffu, him, o);
    }
    if (lane == 0) {
        Hb[e] = make_double2(hre, him);
        if (l == 0) Sb[r] = make_double2(s, 0.0);
    }
}

// Splits the complex FP64 bands into FP32 pairs (re hi, re lo, im hi, im lo)
// for the mixed assembly, and reduces the smallest and largest non-zero
// magnitude of the real and imaginary parts into range[0..1] (bit patterns of
// positive doubles order like integers); the host enables the FP32-pair
// products only if every product of two band values, and its TwoProd error
// terms, stays normal FP32.
__global__ void k_band_split(const double2 *__restrict__ src, int64_t n, float4 *__restrict__ dst,
                             unsigned long long *__restrict__ range) {
    unsigned long long mn = 0x7ff0000000000000ull, mx = 0ull;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x) {
        double2 v = src[e];
        float rh = __double2float_rn(v.x), ih = __double2float_rn(v.y);
        float rl = __double2float_rn(v.x - (double)rh), il = __double2float_rn(v.y - (double)ih);
        dst[e] = make_float4(rh, rl, ih, il);
        const unsigned long long br = (unsigned long long)__double_as_longlong(fabs(v.x));
        const unsigned long long bi = (unsigned long long)__double_as_longlong(fabs(v.y));
        if (br) {
            mn = min(mn, br);
            mx = max(mx, br);
        }
        if (bi) {
            mn = min(mn, bi);
            mx = max(mx, bi);
        }
    }
    if (mx) {
        atomicMin(&range[0], mn);
        atomicMax(&range[1], mx);
    }
}

}  // namespace

static inline unsigned grid_for(int64_t n, int threads) {
    int64_t g = (n + threads - 1) / threads;
    if (g > (int64_t)152 * 64) g = (int64_t)152 * 64;
    if (g < 1) g = 1;
    return (unsigned)g;
}

RadialDev radial_dev(const bs2e_handle *h) {
    const Radial &g = h->g;
    RadialDev P;
    P.knots = h->d_knots;
    P.glx = h->d_glx;
    P.glw = h->d_glw;
    P.tab_r = h->d_tab_r;
    P.tab_B = h->d_tab_B;
    P.tab_D2 = h->d_tab_D2;
    P.tab_D1 = h->d_tab_D1;
    P.tab_ri = h->d_tab_ri;
    P.tab_Bi = h->d_tab_Bi;
    P.mom = h->d_mom;
    P.dint = h->d_dint;
    P.dsym = h->d_dsym;
    P.tot = h->d_tot;
    P.R = h->d_R;
    P.Rf = h->d_Rf;
    P.Rexp = h->d_Rexp;
    P.k = g.k;
    P.q = g.q;
    P.K1 = g.K1;
    P.N = g.N;
    P.n_iv = g.n_iv;
    P.mixed = h->precision == BS2E_PREC_MIXED ? 1 : 0;
    P.tile = g.tile;
    return P;
}

void launch_tabulate(bs2e_handle *h) {
    const Radial &g = h->g;
    // several CTAs per interval: each de Boor evaluation is a long serial chain
    // of FP64 divisions, so the launch needs many resident warps
    const int parts = std::max(1, std::min(8, (g.q * g.q * g.k + 127) / 128));
    k_tabulate<<<dim3((unsigned)g.n_iv, (unsigned)parts), 128, 0, h->stream>>>(radial_dev(h));
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
    k_moments<<<grid, 256, smem, h->stream>>>(radial_dev(h));
    h->launches++;
}

void launch_totals(bs2e_handle *h) {
    const Radial &g = h->g;
    int64_t n = (int64_t)2 * g.K1 * g.N * g.W;
    k_totals<<<grid_for(n, 256), 256, 0, h->stream>>>(radial_dev(h));
    h->launches++;
}

size_t rk_store_smem(const Radial &g, bool mixed) {
    return sizeof(double) * (rk_scratch(g.k, g.K1) + (mixed ? (size_t)g.K1 * g.W * g.W : 0));
}

void launch_rk_fill(bs2e_handle *h, int k_first, int k_count) {
    const Radial &g = h->g;
    unsigned tiles = (unsigned)((int64_t)g.N * g.N);
    const bool mixed = h->precision == BS2E_PREC_MIXED;
    const size_t smem = rk_store_smem(g, mixed);
    if (mixed) {
        cudaFuncSetAttribute(k_rk_store_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_rk_store_mixed<<<tiles, 256, smem, h->stream>>>(radial_dev(h), k_first, k_count);
    } else {
        cudaFuncSetAttribute(k_rk_store, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_rk_store<<<tiles, 256, smem, h->stream>>>(radial_dev(h), k_first, k_count);
    }
    h->launches++;
}

static const void *batch_kernel(int stage) {
    switch (stage) {
        case 0: return (const void *)k_radial_batch<0>;
        case 1: return (const void *)k_radial_batch<1>;
        case 2: return (const void *)k_radial_batch<2>;
        case 3: return (const void *)k_radial_batch_rk<3>;
        default: return (const void *)k_radial_batch_rk<4>;
    }
}

int radial_batch_blocks_per_sm(int stage, int threads, size_t smem) {
    cudaFuncSetAttribute(batch_kernel(stage), cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_kernel(stage), threads, smem) !=
        cudaSuccess)
        return 0;
    return nb;
}

void launch_radial_batch(cudaStream_t s, int stage, int grid, int threads, size_t smem,
                         const RadialDev *probs, const int64_t *off, int n,
                         unsigned long long *counter, int chunk, int persistent) {
    BatchStage B;
    B.probs = probs;
    B.off = off;
    B.n = n;
    B.chunk = chunk;
    B.persistent = persistent;
    B.counter = counter;
    switch (stage) {
        case 0: k_radial_batch<0><<<grid, threads, smem, s>>>(B); break;
        case 1: k_radial_batch<1><<<grid, threads, smem, s>>>(B); break;
        case 2: k_radial_batch<2><<<grid, threads, smem, s>>>(B); break;
        case 3: k_radial_batch_rk<3><<<grid, threads, smem, s>>>(B); break;
        default: k_radial_batch_rk<4><<<grid, threads, smem, s>>>(B); break;
    }
}

void launch_rk_gather(bs2e_handle *h, int64_t n, const int64_t *d_keys, double *d_vals) {
    const Radial &g = h->g;
    k_rk_gather<<<grid_for(n * g.K1, 256), 256, 0, h->stream>>>(
        h->d_R, h->d_Rf, h->d_Rexp, g.k, g.K1, g.N, g.tile, n, d_keys, d_vals);
    h->launches++;
}

void launch_rk_slice(bs2e_handle *h, int kk, double *d_out) {
    const Radial &g = h->g;
    const int64_t n = (int64_t)g.N * g.N * g.W * g.W;
    const bool mixed = h->precision == BS2E_PREC_MIXED;
    k_rk_slice<<<grid_for(n, 256), 256, 0, h->stream>>>(mixed ? nullptr : h->d_R, h->d_Rf,
                                                        h->d_Rexp, kk, g.k, g.K1, g.N, g.tile,
                                                        d_out);
    h->launches++;
}

void launch_band_split(bs2e_handle *h) {
    const Radial &g = h->g;
    int64_t nh = h->n_l * g.N * g.W, ns = (int64_t)g.N * g.W;
    const unsigned long long init[4] = {0x7ff0000000000000ull, 0ull, 0x7ff0000000000000ull, 0ull};
    cudaMemcpyAsync(h->d_range, init, sizeof(init), cudaMemcpyHostToDevice, h->stream);
    k_band_split<<<grid_for(nh, 256), 256, 0, h->stream>>>(h->d_Hb, nh, h->d_Hbf, h->d_range);
    k_band_split<<<grid_for(ns, 256), 256, 0, h->stream>>>(h->d_Sb, ns, h->d_Sbf, h->d_range + 2);
    cudaStreamSynchronize(h->stream);  // init lives on this stack frame
    h->launches += 2;
}

void launch_one_body(bs2e_handle *h, int64_t Z, int64_t n_l, int64_t cap_order, double cap_r0,
                     double eta_re, double eta_im) {
    const Radial &g = h->g;
    int64_t n = n_l * g.N * g.W;
    k_one_body<<<(unsigned)((n * 32 + 127) / 128), 128, 0, h->stream>>>(
        h->d_knots, h->d_glw, h->d_tab_r, h->d_tab_B, h->d_tab_D2, g.k, g.q, g.N, g.n_iv, (int)Z,
        (int)n_l, (int)cap_order, cap_r0, eta_re, eta_im, h->d_Sb, h->d_Hb);
    h->launches++;
}

}  // namespace bs2e
