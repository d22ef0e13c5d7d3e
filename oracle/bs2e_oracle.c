/*
 * bs2e_oracle.c -- CPU oracle (test infrastructure only) for the two-electron
 * matrix-element path of edvinolo/b-spline-two-e.
 *
 * Each function restates one routine of the reference Fortran, with the same
 * loop order, thresholds and accumulation order, and cites the file:line it
 * follows.  Two third-party routines sit on the path and are restated from
 * their published algorithms:
 *   - fortran-lang/stdlib gauss_legendre (Newton on P_n from Gauss-Chebyshev
 *     guesses), called at src/tools/quad_tools.f90:26; version unpinned by the
 *     reference (git HEAD clone, utils/install_bs2e_aws_linux_2023.sh:72);
 *   - GSL gsl_sf_coupling_3j / gsl_sf_coupling_6j, called at
 *     src/tools/wigner_tools.f90:43,59; version unpinned (distro gsl-devel).
 *     Restated here as the Racah single-sum formulas in long double.
 * Neither boundary is pinned by the reference's own tests (they only print),
 * so tests/ pin these against exact sympy values and numpy's leggauss.
 *
 * Build with -ffp-contract=off so results do not depend on whether the host
 * compiler fuses multiply-adds (x86-64 vs aarch64).
 */
#include "bs2e_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* Gauss-Legendre (stdlib gauss_legendre as used by quad_tools.f90:14-27)    */
/* ------------------------------------------------------------------------ */

static double leg_p(int64_t n, double x) {
    if (n == 0) return 1.0;
    if (n == 1) return x;
    double p2 = 1.0, p1 = x, p = x;
    for (int64_t i = 2; i <= n; ++i) {
        p = (double)(2 * i - 1) * x * p1 / (double)i - (double)(i - 1) * p2 / (double)i;
        p2 = p1;
        p1 = p;
    }
    return p;
}

static double leg_dp(int64_t n, double x) {
    if (n == 0) return 0.0;
    if (n == 1) return 1.0;
    double p2 = 1.0, p1 = x, d2 = 0.0, d1 = 1.0, p = x, d = 1.0;
    for (int64_t i = 2; i <= n; ++i) {
        p = (double)(2 * i - 1) * x * p1 / (double)i - (double)(i - 1) * p2 / (double)i;
        d = d2 + (double)(2 * i - 1) * p1;
        p2 = p1;
        p1 = p;
        d2 = d1;
        d1 = d;
    }
    return d;
}

void or_gauss_legendre(int64_t q, double *x, double *w) {
    const double pi = 3.14159265358979323846264338327950288;
    int64_t n = q - 1;
    if (n == 0) {
        x[0] = 0.0;
        w[0] = 2.0;
        return;
    }
    if (n == 1) {
        x[0] = -sqrt(1.0 / 3.0);
        x[1] = -x[0];
        w[0] = w[1] = 1.0;
        return;
    }
    const double tol = 4.0 * 2.220446049250313e-16;
    for (int64_t i = 0; i <= (n + 1) / 2 - 1; ++i) {
        double xi = -cos((double)(2 * i + 1) / (2.0 * (double)n + 2.0) * pi);
        for (int it = 0; it < 100; ++it) {
            double delta = -leg_p(n + 1, xi) / leg_dp(n + 1, xi);
            xi += delta;
            if (fabs(delta) <= tol * fabs(xi)) break;
        }
        x[i] = xi;
        x[n - i] = -xi;
        double dl = leg_dp(n + 1, xi);
        w[i] = 2.0 / ((1.0 - xi * xi) * dl * dl);
        w[n - i] = w[i];
    }
    if (n % 2 == 0) {
        x[n / 2] = 0.0;
        double dl = leg_dp(n + 1, 0.0);
        w[n / 2] = 2.0 / (dl * dl);
    }
}

/* ------------------------------------------------------------------------ */
/* B-splines (src/tools/bspline_tools.f90)                                   */
/* ------------------------------------------------------------------------ */

/* BVALUE_D with the interval hint (bspline_tools.f90:151-224); the coefficient
 * vector is the unit vector of spline jspline (the reference's c_i/c_j). */
double or_bvalue(const double *t, int64_t n, int64_t k, double x, int64_t ideriv, int64_t iv,
                 int64_t jspline) {
    (void)n;
    double aj[22], dpv[22], dmv[22];
    int64_t kmd = k - ideriv;
    if (kmd <= 0) return 0.0;
    int64_t km1 = k - 1;
    int64_t i = k - 1 + iv; /* 1-based left knot of the interval */
#define T(idx) t[(idx)-1]
    for (int64_t j = 1; j <= k; ++j) aj[j] = (i - k + j == jspline) ? 1.0 : 0.0;
    for (int64_t j = 1; j <= ideriv; ++j) {
        int64_t kmj = k - j;
        for (int64_t jj = 1; jj <= kmj; ++jj) {
            int64_t ihi = i + jj;
            int64_t ihmkmj = ihi - kmj;
            aj[jj] = (aj[jj + 1] - aj[jj]) / (T(ihi) - T(ihmkmj)) * (double)kmj;
        }
    }
    for (int64_t j = 1; j <= kmd; ++j) {
        dpv[j] = T(i + j) - x;
        dmv[j] = x - T(i + 1 - j);
    }
    for (int64_t j = ideriv + 1; j <= km1; ++j) {
        int64_t kmj = k - j;
        int64_t ii = kmj;
        for (int64_t jj = 1; jj <= kmj; ++jj) {
            aj[jj] = (aj[jj + 1] * dmv[ii] + aj[jj] * dpv[jj]) / (dmv[ii] + dpv[jj]);
            ii -= 1;
        }
    }
#undef T
    return aj[1];
}

/* support(iv, jf): interval iv (1-based) lies in the support of full spline jf
 * (bspline_tools.f90:42-56). */
static inline int supp(int64_t iv, int64_t jf, int64_t k) { return iv <= jf && jf <= iv + k - 1; }

/* ------------------------------------------------------------------------ */
/* 3j / 6j (GSL coupling, restated as Racah's formulas)                       */
/* ------------------------------------------------------------------------ */

static long double lfact(int64_t m) {
    static long double tab[200];
    static int init = 0;
    if (!init) {
        long double f = 1.0L;
        tab[0] = 1.0L;
        for (int i = 1; i < 200; ++i) {
            f *= (long double)i;
            tab[i] = f;
        }
        init = 1;
    }
    return tab[m];
}

static int tri_ok(int64_t a, int64_t b, int64_t c) {
    return a >= 0 && b >= 0 && c >= 0 && c <= a + b && c >= (a > b ? a - b : b - a);
}

static long double delta_tri(int64_t a, int64_t b, int64_t c) {
    return sqrtl(lfact(a + b - c) * lfact(a - b + c) * lfact(-a + b + c) / lfact(a + b + c + 1));
}

double or_three_j(int64_t j1, int64_t j2, int64_t j3, int64_t m1, int64_t m2, int64_t m3) {
    if (m1 + m2 + m3 != 0) return 0.0;
    if (!tri_ok(j1, j2, j3)) return 0.0;
    if (llabs(m1) > j1 || llabs(m2) > j2 || llabs(m3) > j3) return 0.0;
    int64_t tmin = 0, tmax = j1 + j2 - j3;
    if (j2 - j3 - m1 > tmin) tmin = j2 - j3 - m1;
    if (j1 - j3 + m2 > tmin) tmin = j1 - j3 + m2;
    if (j1 - m1 < tmax) tmax = j1 - m1;
    if (j2 + m2 < tmax) tmax = j2 + m2;
    long double s = 0.0L;
    for (int64_t t = tmin; t <= tmax; ++t) {
        long double den = lfact(t) * lfact(j3 - j2 + t + m1) * lfact(j3 - j1 + t - m2) *
                          lfact(j1 + j2 - j3 - t) * lfact(j1 - t - m1) * lfact(j2 - t + m2);
        s += ((t & 1) ? -1.0L : 1.0L) / den;
    }
    long double pre = delta_tri(j1, j2, j3) *
                      sqrtl(lfact(j1 + m1) * lfact(j1 - m1) * lfact(j2 + m2) * lfact(j2 - m2) *
                            lfact(j3 + m3) * lfact(j3 - m3));
    int64_t ph = j1 - j2 - m3;
    long double sg = (llabs(ph) & 1) ? -1.0L : 1.0L;
    return (double)(sg * pre * s);
}

double or_six_j(int64_t j1, int64_t j2, int64_t j3, int64_t j4, int64_t j5, int64_t j6) {
    if (!tri_ok(j1, j2, j3) || !tri_ok(j1, j5, j6) || !tri_ok(j4, j2, j6) || !tri_ok(j4, j5, j3))
        return 0.0;
    int64_t a1 = j1 + j2 + j3, a2 = j1 + j5 + j6, a3 = j4 + j2 + j6, a4 = j4 + j5 + j3;
    int64_t b1 = j1 + j2 + j4 + j5, b2 = j2 + j3 + j5 + j6, b3 = j3 + j1 + j6 + j4;
    int64_t tmin = a1;
    if (a2 > tmin) tmin = a2;
    if (a3 > tmin) tmin = a3;
    if (a4 > tmin) tmin = a4;
    int64_t tmax = b1;
    if (b2 < tmax) tmax = b2;
    if (b3 < tmax) tmax = b3;
    long double s = 0.0L;
    for (int64_t t = tmin; t <= tmax; ++t) {
        long double den = lfact(t - a1) * lfact(t - a2) * lfact(t - a3) * lfact(t - a4) *
                          lfact(b1 - t) * lfact(b2 - t) * lfact(b3 - t);
        s += ((t & 1) ? -1.0L : 1.0L) * lfact(t + 1) / den;
    }
    long double pre = delta_tri(j1, j2, j3) * delta_tri(j1, j5, j6) * delta_tri(j4, j2, j6) *
                      delta_tri(j4, j5, j3);
    return (double)(pre * s);
}

/* C_red_mat (wigner_tools.f90:107-112). */
double or_C_red_mat(int64_t k, int64_t a, int64_t b) {
    double sg = (a & 1) ? -1.0 : 1.0;
    return sg * sqrt((double)((2 * a + 1) * (2 * b + 1))) * or_three_j(a, k, b, 0, 0, 0);
}

/* ang_k_LS (wigner_tools.f90:126-138). confs(1)=(la,lb), confs(2)=(lc,ld). */
double or_ang_k_LS(int64_t k, int64_t la, int64_t lb, int64_t lc, int64_t ld, int64_t L) {
    if (((la + k + lc) % 2) != 0 || ((lb + k + ld) % 2) != 0) return 0.0;
    double sg = ((lb + lc + L) & 1) ? -1.0 : 1.0;
    return sg * or_six_j(la, lb, L, ld, lc, k) * or_C_red_mat(k, la, lc) * or_C_red_mat(k, lb, ld);
}

/* ------------------------------------------------------------------------ */
/* COO counts (sparse_array_tools.f90:276-324)                               */
/* ------------------------------------------------------------------------ */

int64_t or_nnz4(int64_t n_knots, int64_t k) {
    int64_t n = n_knots - k, nb = n - 2, n_iv = n_knots - 2 * k + 1;
    int64_t nnz = 0;
    for (int64_t j = 1; j <= nb; ++j)
        for (int64_t i = 1; i <= nb; ++i) {
            if (llabs(i - j) >= k) continue;
            for (int64_t iv = 1; iv <= n_iv; ++iv)
                if (supp(iv, i + 1, k) && supp(iv, j + 1, k)) nnz++;
        }
    return nnz;
}

int64_t or_nnz6(int64_t n_knots, int64_t k) {
    int64_t n = n_knots - k, nb = n - 2, n_iv = n_knots - 2 * k + 1;
    int64_t nnz = 0;
    for (int64_t jp = 1; jp <= nb; ++jp)
        for (int64_t j = 1; j <= nb; ++j) {
            if (llabs(j - jp) >= k) continue;
            for (int64_t ip = 1; ip <= nb; ++ip)
                for (int64_t i = 1; i <= nb; ++i) {
                    if (llabs(i - ip) >= k) continue;
                    for (int64_t iv = 1; iv <= n_iv; ++iv)
                        if (supp(iv, i + 1, k) && supp(iv, ip + 1, k) && supp(iv, j + 1, k) &&
                            supp(iv, jp + 1, k))
                            nnz++;
                }
        }
    return nnz;
}

/* ------------------------------------------------------------------------ */
/* Slater primitives (mat_els.f90:172-292, 392-491)                           */
/* ------------------------------------------------------------------------ */

/* Real ** integer as libgfortran's pow_r8_i8: binary powering. */
static double powi(double a, int64_t b) {
    double pow = 1.0, x = a;
    uint64_t u;
    if (b == 0) return 1.0;
    if (b < 0) {
        u = (uint64_t)(-b);
        x = 1.0 / x;
    } else {
        u = (uint64_t)b;
    }
    for (;;) {
        if (u & 1) pow *= x;
        u >>= 1;
        if (u)
            x *= x;
        else
            break;
    }
    return pow;
}

void or_slater(const double *knots, int64_t n_knots, int64_t k, int64_t k_GL, int64_t max_k,
               double *rk, double *rmk, int64_t *idx4, double *rdk, int64_t *idx6, int nthreads) {
    int64_t n = n_knots - k, nb = n - 2, n_iv = n_knots - 2 * k + 1;
    const double *bp = knots + (k - 1); /* breakpoints(1..n_iv+1) = t(k..n+1) */
    double x[64], w[64];
    or_gauss_legendre(k_GL, x, w);
    int64_t nnz4 = or_nnz4(n_knots, k), nnz6 = or_nnz6(n_knots, k);
    if (nthreads <= 0) {
#ifdef _OPENMP
        nthreads = omp_get_max_threads();
#else
        nthreads = 1;
#endif
    }

    /* setup_Slater_off_diag (mat_els.f90:184-228): OpenMP over k. */
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int64_t kk = 0; kk <= max_k; ++kk) {
        int64_t ptr = 0;
        double r[64], Bi[64], Bj[64];
        for (int64_t jb = 1; jb <= nb; ++jb)
            for (int64_t ib = 1; ib <= nb; ++ib) {
                if (llabs(jb - ib) >= k) continue;
                for (int64_t ir = 1; ir <= n_iv; ++ir) {
                    if (!(supp(ir, ib + 1, k) && supp(ir, jb + 1, k))) continue;
                    ptr++;
                    double lo = bp[ir - 1], hi = bp[ir];
                    /* compute_Slater_off_diag (mat_els.f90:392-439) */
                    double scale = 0.5 * (hi - lo), translate = 0.5 * (hi + lo);
                    for (int64_t s = 0; s < k_GL; ++s) {
                        r[s] = scale * x[s] + translate;
                        Bi[s] = or_bvalue(knots, n, k, r[s], 0, ir, ib + 1);
                        Bj[s] = or_bvalue(knots, n, k, r[s], 0, ir, jb + 1);
                    }
                    double a = 0.0, b = 0.0;
                    for (int64_t s = 0; s < k_GL; ++s) {
                        a = a + w[s] * Bi[s] * Bj[s] * powi(r[s], kk);
                        b = b + w[s] * Bi[s] * Bj[s] / powi(r[s], kk + 1);
                    }
                    rk[(ptr - 1) + nnz4 * kk] = scale * a;
                    rmk[(ptr - 1) + nnz4 * kk] = scale * b;
                    if (kk == 0) {
                        idx4[3 * (ptr - 1) + 0] = ir;
                        idx4[3 * (ptr - 1) + 1] = ib;
                        idx4[3 * (ptr - 1) + 2] = jb;
                    }
                }
            }
    }

    /* setup_Slater_diag (mat_els.f90:230-292): OpenMP over k. */
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int64_t kk = 0; kk <= max_k; ++kk) {
        int64_t ptr = 0;
        double r[64], Bi[64], Bip[64];
        for (int64_t jbp = 1; jbp <= nb; ++jbp)
            for (int64_t jb = 1; jb <= nb; ++jb) {
                if (llabs(jb - jbp) >= k) continue;
                for (int64_t ibp = 1; ibp <= nb; ++ibp)
                    for (int64_t ib = 1; ib <= nb; ++ib) {
                        if (llabs(ib - ibp) >= k) continue;
                        for (int64_t ir = 1; ir <= n_iv; ++ir) {
                            int isup = supp(ir, ib + 1, k) && supp(ir, ibp + 1, k);
                            int jsup = supp(ir, jb + 1, k) && supp(ir, jbp + 1, k);
                            if (!(isup && jsup)) continue;
                            ptr++;
                            double lo = bp[ir - 1], hi = bp[ir];
                            /* compute_Slater_diag (mat_els.f90:441-491) */
                            double sci = 0.5 * (hi - lo), tri = 0.5 * (hi + lo);
                            for (int64_t s = 0; s < k_GL; ++s) {
                                r[s] = sci * x[s] + tri;
                                Bi[s] = or_bvalue(knots, n, k, r[s], 0, ir, ib + 1);
                                Bip[s] = or_bvalue(knots, n, k, r[s], 0, ir, ibp + 1);
                            }
                            double acc = 0.0;
                            for (int64_t s = 0; s < k_GL; ++s) {
                                double scj = 0.5 * (r[s] - lo), trj = 0.5 * (r[s] + lo);
                                double intj = 0.0;
                                for (int64_t u = 0; u < k_GL; ++u) {
                                    double rj = scj * x[u] + trj;
                                    double Bj = or_bvalue(knots, n, k, rj, 0, ir, jb + 1);
                                    double Bjp = or_bvalue(knots, n, k, rj, 0, ir, jbp + 1);
                                    intj = intj + w[u] * Bj * Bjp * powi(rj, kk);
                                }
                                intj = scj * intj;
                                acc = acc + w[s] * Bi[s] * Bip[s] * intj / powi(r[s], kk + 1);
                            }
                            rdk[(ptr - 1) + nnz6 * kk] = sci * acc;
                            if (kk == 0) {
                                int64_t *e = idx6 + 5 * (ptr - 1);
                                e[0] = ir;
                                e[1] = ib;
                                e[2] = ibp;
                                e[3] = jb;
                                e[4] = jbp;
                            }
                        }
                    }
            }
    }
}

/* ------------------------------------------------------------------------ */
/* R^k map (sparse_array_tools.f90:452-493, set_val :509-534)                 */
/* ------------------------------------------------------------------------ */

static inline size_t rk_key(int64_t nb, int64_t k, int64_t K1, int64_t a, int64_t b, int64_t c,
                            int64_t d) {
    int64_t W = 2 * k - 1;
    return ((((size_t)(a - 1) * nb + (size_t)(b - 1)) * W + (size_t)(c - a + k - 1)) * W +
            (size_t)(d - b + k - 1)) *
           (size_t)K1;
}

void or_rk_map(int64_t n_b, int64_t k, int64_t max_k, int64_t nnz4, const double *rk,
               const double *rmk, const int64_t *idx4, int64_t nnz6, const double *rdk,
               const int64_t *idx6, double *R) {
    int64_t K1 = max_k + 1, W = 2 * k - 1;
    memset(R, 0, sizeof(double) * (size_t)n_b * n_b * W * W * K1);
    /* Serial double loop over all pairs of interval moments, as the reference. */
    for (int64_t n = 0; n < nnz4; ++n) {
        int64_t ivn = idx4[3 * n], in = idx4[3 * n + 1], jn = idx4[3 * n + 2];
        for (int64_t m = 0; m < nnz4; ++m) {
            int64_t ivm = idx4[3 * m], im = idx4[3 * m + 1], jm = idx4[3 * m + 2];
            if (ivn == ivm) continue;
            double *dst = R + rk_key(n_b, k, K1, in, im, jn, jm);
            if (ivn < ivm) {
                for (int64_t kk = 0; kk < K1; ++kk)
                    dst[kk] = dst[kk] + rk[n + nnz4 * kk] * rmk[m + nnz4 * kk];
            } else {
                for (int64_t kk = 0; kk < K1; ++kk)
                    dst[kk] = dst[kk] + rk[m + nnz4 * kk] * rmk[n + nnz4 * kk];
            }
        }
    }
    for (int64_t n = 0; n < nnz6; ++n) {
        const int64_t *e = idx6 + 5 * n; /* iv, i, i_p, j, j_p */
        double *d1 = R + rk_key(n_b, k, K1, e[1], e[3], e[2], e[4]);
        for (int64_t kk = 0; kk < K1; ++kk) d1[kk] = d1[kk] + rdk[n + nnz6 * kk];
        double *d2 = R + rk_key(n_b, k, K1, e[3], e[1], e[4], e[2]);
        for (int64_t kk = 0; kk < K1; ++kk) d2[kk] = d2[kk] + rdk[n + nnz6 * kk];
    }
}

/* ------------------------------------------------------------------------ */
/* R^k of selected tiles, for bases where the full primitives are too slow    */
/* ------------------------------------------------------------------------ */

/* Spline values of one breakpoint interval at or_slater's quadrature points:
 * outer radii r[s] and, for each s, the inner radii rj[s][u] of the kink-split
 * integral on [lo, r[s]]; B[s][f] / Bj[s][u][f] hold full spline ir + f
 * (f < k), the only ones non-zero on the interval.  Same expressions as
 * or_slater, so every cached value is the one or_slater computes. */
typedef struct {
    int64_t ir;
    double lo, hi;
    double *r, *B, *rj, *Bj;
} iv_cache;

static void iv_cache_fill(iv_cache *c, const double *knots, int64_t n, int64_t k, int64_t q,
                          const double *x, int64_t ir) {
    const double *bp = knots + (k - 1);
    c->ir = ir;
    c->lo = bp[ir - 1];
    c->hi = bp[ir];
    double scale = 0.5 * (c->hi - c->lo), translate = 0.5 * (c->hi + c->lo);
    for (int64_t s = 0; s < q; ++s) {
        double rs = scale * x[s] + translate;
        c->r[s] = rs;
        for (int64_t f = 0; f < k; ++f) c->B[s * k + f] = or_bvalue(knots, n, k, rs, 0, ir, ir + f);
        double scj = 0.5 * (rs - c->lo), trj = 0.5 * (rs + c->lo);
        for (int64_t u = 0; u < q; ++u) {
            double rj = scj * x[u] + trj;
            c->rj[s * q + u] = rj;
            for (int64_t f = 0; f < k; ++f)
                c->Bj[(s * q + u) * k + f] = or_bvalue(knots, n, k, rj, 0, ir, ir + f);
        }
    }
}

/* Entry v of a tile's interval cache, filled on first use. */
static const iv_cache *ivc_get(iv_cache *cache, double **mem, int64_t v, size_t per,
                               const double *knots, int64_t n, int64_t k, int64_t q,
                               const double *x, int64_t ir) {
    iv_cache *c = &cache[v];
    if (!mem[v]) {
        double *m = (double *)malloc(sizeof(double) * per);
        mem[v] = m;
        c->r = m;
        c->B = m + q;
        c->rj = m + q + q * k;
        c->Bj = m + q + q * k + q * q;
        iv_cache_fill(c, knots, n, k, q, x, ir);
    }
    return c;
}

/* r_k / r_m_k of basis pair (ib, jb) on interval c->ir for multipole kk:
 * compute_Slater_off_diag (mat_els.f90:392-439) as or_slater evaluates it. */
static void prim_off(const iv_cache *c, int64_t k, int64_t q, const double *w, int64_t ib,
                     int64_t jb, int64_t kk, double *rk, double *rmk) {
    double scale = 0.5 * (c->hi - c->lo);
    int64_t fi = ib + 1 - c->ir, fj = jb + 1 - c->ir;
    double a = 0.0, b = 0.0;
    for (int64_t s = 0; s < q; ++s) {
        double Bi = c->B[s * k + fi], Bj = c->B[s * k + fj];
        a = a + w[s] * Bi * Bj * powi(c->r[s], kk);
        b = b + w[s] * Bi * Bj / powi(c->r[s], kk + 1);
    }
    *rk = scale * a;
    *rmk = scale * b;
}

/* r_d_k of (ib, ibp; jb, jbp) on interval c->ir for multipole kk:
 * compute_Slater_diag (mat_els.f90:441-491) as or_slater evaluates it. */
static double prim_diag(const iv_cache *c, int64_t k, int64_t q, const double *w, int64_t ib,
                        int64_t ibp, int64_t jb, int64_t jbp, int64_t kk) {
    double sci = 0.5 * (c->hi - c->lo);
    int64_t fi = ib + 1 - c->ir, fip = ibp + 1 - c->ir, fj = jb + 1 - c->ir,
            fjp = jbp + 1 - c->ir;
    double acc = 0.0;
    for (int64_t s = 0; s < q; ++s) {
        double scj = 0.5 * (c->r[s] - c->lo);
        double intj = 0.0;
        for (int64_t u = 0; u < q; ++u) {
            const double *Bu = c->Bj + (s * q + u) * k;
            intj = intj + w[u] * Bu[fj] * Bu[fjp] * powi(c->rj[s * q + u], kk);
        }
        intj = scj * intj;
        acc = acc + w[s] * c->B[s * k + fi] * c->B[s * k + fip] * intj / powi(c->r[s], kk + 1);
    }
    return sci * acc;
}

/* Intervals (1-based, ascending) where basis splines i and j are both
 * non-zero: support(ir, i+1) and support(ir, j+1), clipped to 1..n_iv. */
static void pair_ivs(int64_t i, int64_t j, int64_t k, int64_t n_iv, int64_t *lo, int64_t *hi) {
    int64_t mx = i > j ? i : j, mn = i < j ? i : j;
    *lo = mx + 2 - k < 1 ? 1 : mx + 2 - k;
    *hi = mn + 1 > n_iv ? n_iv : mn + 1;
}

void or_rk_tiles(const double *knots, int64_t n_knots, int64_t k, int64_t k_GL, int64_t max_k,
                 int64_t n_tiles, const int64_t *ab, double *out, int nthreads) {
    int64_t n = n_knots - k, nb = n - 2, n_iv = n_knots - 2 * k + 1;
    int64_t K1 = max_k + 1, W = 2 * k - 1, q = k_GL;
    double x[64], w[64];
    or_gauss_legendre(q, x, w);
    if (nthreads <= 0) {
#ifdef _OPENMP
        nthreads = omp_get_max_threads();
#else
        nthreads = 1;
#endif
    }
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int64_t t = 0; t < n_tiles; ++t) {
        const int64_t a = ab[2 * t], b = ab[2 * t + 1];
        double *o = out + (size_t)t * W * W * K1;
        memset(o, 0, sizeof(double) * (size_t)W * W * K1);
        /* intervals the pairs (a, c) and (b, d) of the tile can share:
         * [a + 2 - k, a + 1] and [b + 2 - k, b + 1], filled on first use */
        int64_t lo = (a < b ? a : b) + 2 - k, hi = (a > b ? a : b) + 1;
        if (lo < 1) lo = 1;
        if (hi > n_iv) hi = n_iv;
        int64_t niv = hi - lo + 1;
        const size_t per = (size_t)(q + q * k + q * q + q * q * k);
        iv_cache *cache = (iv_cache *)calloc((size_t)niv, sizeof(iv_cache));
        double **mem = (double **)calloc((size_t)niv, sizeof(double *));
#define IVC(ir) ivc_get(cache, mem, (ir) - lo, per, knots, n, k, q, x, (ir))
        for (int64_t dc = 0; dc < W; ++dc) {
            const int64_t c = a + dc - (k - 1);
            if (c < 1 || c > nb) continue;
            for (int64_t dd = 0; dd < W; ++dd) {
                const int64_t d = b + dd - (k - 1);
                if (d < 1 || d > nb) continue;
                double *v = o + ((size_t)dc * W + (size_t)dd) * K1;
                int64_t l1, h1, l2, h2;
                pair_ivs(a, c, k, n_iv, &l1, &h1);
                pair_ivs(b, d, k, n_iv, &l2, &h2);
                /* 4d part: n over the (a, c) entries, m over the (b, d) entries,
                 * both by ascending interval (or_rk_map's loop order) */
                for (int64_t kk = 0; kk < K1; ++kk) {
                    double acc = 0.0;
                    for (int64_t iv1 = l1; iv1 <= h1; ++iv1) {
                        double rk1, rmk1;
                        prim_off(IVC(iv1), k, q, w, a, c, kk, &rk1, &rmk1);
                        for (int64_t iv2 = l2; iv2 <= h2; ++iv2) {
                            if (iv1 == iv2) continue;
                            double rk2, rmk2;
                            prim_off(IVC(iv2), k, q, w, b, d, kk, &rk2, &rmk2);
                            if (iv1 < iv2)
                                acc = acc + rk1 * rmk2;
                            else
                                acc = acc + rk2 * rmk1;
                        }
                    }
                    v[kk] = acc;
                }
                /* 6d part: entries (ir; ib=a, ibp=c, jb=b, jbp=d) add through
                 * their direct key, entries (ir; ib=b, ibp=d, jb=a, jbp=c)
                 * through their swapped key; in the 6d COO order (jbp, jb,
                 * ibp, ib, ir) one group precedes the other, or both are the
                 * same entries (a = b, c = d), each adding twice */
                int64_t s_lo = l1 > l2 ? l1 : l2, s_hi = h1 < h2 ? h1 : h2;
                int same = (a == b && c == d);
                int direct_first = (d < c) || (d == c && (b < a || (b == a && (c < d || (c == d && a < b)))));
                for (int g = 0; g < 2; ++g) {
                    int direct = same ? 1 : (g == 0 ? direct_first : !direct_first);
                    if (same && g == 1) break;
                    for (int64_t ir = s_lo; ir <= s_hi; ++ir) {
                        for (int64_t kk = 0; kk < K1; ++kk) {
                            double dv = direct ? prim_diag(IVC(ir), k, q, w, a, c, b, d, kk)
                                               : prim_diag(IVC(ir), k, q, w, b, d, a, c, kk);
                            v[kk] = v[kk] + dv;
                            if (same) v[kk] = v[kk] + dv;
                        }
                    }
                }
            }
        }
#undef IVC
        for (int64_t v = 0; v < niv; ++v) free(mem[v]);
        free(mem);
        free(cache);
    }
}

/* ------------------------------------------------------------------------ */
/* Basis enumeration (orbital_tools.f90:46-72, 119-216)                       */
/* ------------------------------------------------------------------------ */

/* consistent() with the triplet extension: the reference drops equivalent
 * configurations for odd L (singlet); the triplet drops them for even L. */
static int consistent(int64_t l1, int64_t l2, int64_t L, int64_t parity_odd, int64_t eqv,
                      int64_t spin) {
    if (eqv && ((spin == 0) ? (L % 2 != 0) : (L % 2 == 0))) return 0;
    int tri = (llabs(l1 - l2) <= L) && (L <= l1 + l2);
    if (!tri) return 0;
    int par = ((l1 % 2 != 0) != (l2 % 2 != 0)) == (parity_odd != 0);
    return par;
}

int64_t or_count_configs(int64_t L, int64_t parity_odd, int64_t max_l_1p, int64_t n_b,
                         int64_t k, int64_t max_n_b, int64_t n_all_l, int64_t l2_max,
                         int64_t spin, or_config *out) {
    int64_t cnt = 0;
    for (int64_t i = 0; i <= max_l_1p; ++i)
        for (int64_t j = 0; j <= i; ++j) {
            int64_t ni0 = (i + 1 < k - 1) ? i + 1 : k - 1;
            int64_t nj0 = (j + 1 < k - 1) ? j + 1 : k - 1;
            for (int64_t ni = ni0; ni <= n_b; ++ni) {
                if (ni > n_all_l && j > l2_max) continue;
                int64_t nj1 = (j == i) ? (ni < max_n_b ? ni : max_n_b)
                                       : (n_b < max_n_b ? n_b : max_n_b);
                for (int64_t nj = nj0; nj <= nj1; ++nj) {
                    int64_t eqv = (i == j) && (ni == nj);
                    if (!consistent(i, j, L, parity_odd, eqv, spin)) continue;
                    if (out) {
                        out[cnt].n1 = ni;
                        out[cnt].n2 = nj;
                        out[cnt].l1 = i;
                        out[cnt].l2 = j;
                        out[cnt].eqv = eqv;
                    }
                    cnt++;
                }
            }
        }
    return cnt;
}

/* ------------------------------------------------------------------------ */
/* Block assembly (hamiltonian.f90:106-283, 348-416; mat_els.f90:552-715)     */
/* ------------------------------------------------------------------------ */

/* ang_k_LS memo for one L: pure-function cache over ordered l pairs. */
typedef struct {
    int64_t lmax, K1, L;
    double *v; /* [(la*(lmax+1)+lb)][(lc*(lmax+1)+ld)][k], NAN = not yet computed */
} ang_cache;

static void ang_cache_init(ang_cache *c, int64_t lmax, int64_t K1, int64_t L) {
    c->lmax = lmax;
    c->K1 = K1;
    c->L = L;
    size_t nl = (size_t)(lmax + 1) * (lmax + 1);
    size_t sz = nl * nl * (size_t)K1;
    c->v = (double *)malloc(sizeof(double) * sz);
    for (size_t i = 0; i < sz; ++i) c->v[i] = NAN;
}

static double ang_get(ang_cache *c, int64_t k, int64_t la, int64_t lb, int64_t lc, int64_t ld) {
    int64_t m = c->lmax + 1;
    size_t i = ((size_t)(la * m + lb) * (size_t)(m * m) + (size_t)(lc * m + ld)) * c->K1 + k;
    if (isnan(c->v[i])) c->v[i] = or_ang_k_LS(k, la, lb, lc, ld, c->L);
    return c->v[i];
}

static int64_t lmax_of(const or_config *cf, int64_t n) {
    int64_t m = 0;
    for (int64_t i = 0; i < n; ++i) {
        if (cf[i].l1 > m) m = cf[i].l1;
        if (cf[i].l2 > m) m = cf[i].l2;
    }
    return m;
}

void or_count_nnz(const or_config *cf, int64_t n_config, int64_t L, int64_t spin, int64_t k,
                  int64_t max_k, int64_t full, int64_t *nnz) {
    (void)spin;
    ang_cache ac;
    ang_cache_init(&ac, lmax_of(cf, n_config), max_k + 1, L);
    int64_t res0 = 0, res1 = 0;
    for (int64_t i = 0; i < n_config; ++i) {
        int64_t na = cf[i].n1, nbb = cf[i].n2, la = cf[i].l1, lb = cf[i].l2;
        for (int64_t j = full ? 0 : i; j < n_config; ++j) {
            int64_t nc = cf[j].n1, nd = cf[j].n2, lc = cf[j].l1, ld = cf[j].l2;
            int support = llabs(na - nc) < k && llabs(nbb - nd) < k;
            int support_ex = llabs(na - nd) < k && llabs(nbb - nc) < k;
            if (support) {
                if (la == lc && lb == ld) res1++;
                for (int64_t kk = 0; kk <= max_k; ++kk)
                    if (fabs(ang_get(&ac, kk, la, lb, lc, ld)) > 5e-15) {
                        res0++;
                        break;
                    }
            } else if (support_ex) {
                if (la == ld && lb == lc) res1++;
                for (int64_t kk = 0; kk <= max_k; ++kk)
                    if (fabs(ang_get(&ac, kk, la, lb, ld, lc)) > 5e-15) {
                        res0++;
                        break;
                    }
            }
        }
    }
    free(ac.v);
    nnz[0] = res0;
    nnz[1] = res1;
}

void or_construct_block(const or_config *cf, int64_t n_config, int64_t L, int64_t spin,
                        int64_t k, int64_t n_b, int64_t max_k, int64_t full, const double *R,
                        const double *H1p, int64_t n_l, const double *S, int64_t row_begin,
                        int64_t row_end, int64_t *H_ptr, int64_t *H_idx, double *H_data,
                        double *H_scale, int64_t *S_ptr, int64_t *S_idx, double *S_data,
                        int64_t *nnz_out) {
    or_construct_block_tiles(cf, n_config, L, spin, k, n_b, max_k, full, R, NULL, H1p, n_l, S,
                             row_begin, row_end, H_ptr, H_idx, H_data, H_scale, S_ptr, S_idx,
                             S_data, nnz_out);
}

void or_construct_block_tiles(const or_config *cf, int64_t n_config, int64_t L, int64_t spin,
                              int64_t k, int64_t n_b, int64_t max_k, int64_t full,
                              const double *R, const int64_t *tile_of, const double *H1p,
                              int64_t n_l, const double *S, int64_t row_begin, int64_t row_end,
                              int64_t *H_ptr, int64_t *H_idx, double *H_data, double *H_scale,
                              int64_t *S_ptr, int64_t *S_idx, double *S_data, int64_t *nnz_out) {
    (void)n_l;
    int64_t K1 = max_k + 1, W = 2 * k - 1;
    ang_cache ac;
    ang_cache_init(&ac, lmax_of(cf, n_config), K1, L);
    const double complex *Hc = (const double complex *)H1p;
    const double complex *Sc = (const double complex *)S;
#define SM(r, c) Sc[((c)-1) * n_b + ((r)-1)]
#define HM(l, r, c) Hc[((size_t)(l) * n_b + ((c)-1)) * n_b + ((r)-1)]
    int fill = (H_idx != NULL);
    int64_t rowH = 1, rowS = 1;
    if (fill) {
        H_ptr[0] = 1;
        S_ptr[0] = 1;
    }
    double exsign = (spin != 0) ? -1.0 : 1.0;
    for (int64_t i = row_begin; i < row_end; ++i) {
        int64_t na = cf[i].n1, nbb = cf[i].n2, la = cf[i].l1, lb = cf[i].l2;
        /* this row's R^k tile (a, b) = (na, nbb): banded store or tile table */
        const double *Rt = NULL;
        if (tile_of) {
            int64_t ti = tile_of[(na - 1) * n_b + (nbb - 1)];
            if (ti < 0) {
                free(ac.v);
                nnz_out[0] = -1;
                nnz_out[1] = -1;
                return;
            }
            Rt = R + (size_t)ti * W * W * K1;
        } else {
            Rt = R + rk_key(n_b, k, K1, na, nbb, na - k + 1, nbb - k + 1);
        }
#define RKT(c, d) (Rt + ((size_t)((c) - na + k - 1) * W + (size_t)((d) - nbb + k - 1)) * K1)
        for (int64_t j = full ? 0 : i; j < n_config; ++j) {
            int64_t nc = cf[j].n1, nd = cf[j].n2, lc = cf[j].l1, ld = cf[j].l2;
            int support = llabs(na - nc) < k && llabs(nbb - nd) < k;
            int support_ex = llabs(na - nd) < k && llabs(nbb - nc) < k;
            if (!(support || support_ex)) continue;
            int r12 = 0;
            for (int64_t kk = 0; kk <= max_k; ++kk) {
                double ang = ang_get(&ac, kk, la, lb, lc, ld);
                double angx = ang_get(&ac, kk, la, lb, ld, lc);
                if ((fabs(ang) > 5e-15 && support) || (fabs(angx) > 5e-15 && support_ex)) {
                    r12 = 1;
                    break;
                }
            }
            int l_eq = (la == lc) && (lb == ld);
            int l_eq_ex = (la == ld) && (lb == lc);
            double sgn = (((lc + ld + L) & 1) ? -1.0 : 1.0) * exsign;
            double complex h = 0.0;
            double scale = 0.0;
            if (r12) {
                /* c_mat_neq_tens (mat_els.f90:608-633) with r_12_tens (:552-571) */
                double res = 0.0;
                if (support) {
                    const double *vals = RKT(nc, nd);
                    double r = 0.0;
                    for (int64_t kk = 0; kk <= max_k; ++kk) {
                        double ang = ang_get(&ac, kk, la, lb, lc, ld);
                        if (fabs(ang) < 5e-16) continue;
                        r = r + vals[kk] * ang;
                        scale += fabs(vals[kk] * ang);
                    }
                    res = res + r;
                }
                if (support_ex) {
                    const double *vals = RKT(nd, nc);
                    double r = 0.0;
                    for (int64_t kk = 0; kk <= max_k; ++kk) {
                        double ang = ang_get(&ac, kk, la, lb, ld, lc);
                        if (fabs(ang) < 5e-16) continue;
                        r = r + vals[kk] * ang;
                        scale += fabs(vals[kk] * ang);
                    }
                    res = res + sgn * r;
                }
                h = h + res;
            }
            if ((support && l_eq) || (support_ex && l_eq_ex)) {
                /* H_1p_neq (mat_els.f90:697-715) and S_mat_neq (:664-678) */
                double complex h1 = 0.0, s1 = 0.0;
                if (l_eq) {
                    double complex t1 = HM(la, na, nc) * SM(nbb, nd);
                    double complex t2 = HM(lb, nbb, nd) * SM(na, nc);
                    h1 = h1 + t1 + t2;
                    s1 = s1 + SM(na, nc) * SM(nbb, nd);
                    scale += cabs(t1) + cabs(t2);
                }
                if (l_eq_ex) {
                    double complex t1 = HM(la, na, nd) * SM(nbb, nc);
                    double complex t2 = HM(lb, nbb, nc) * SM(na, nd);
                    h1 = h1 + (t1 + t2) * sgn;
                    s1 = s1 + sgn * SM(na, nd) * SM(nbb, nc);
                    scale += cabs(t1) + cabs(t2);
                }
                h = h + h1;
                if (fill) {
                    S_data[2 * (rowS - 1)] = creal(s1);
                    S_data[2 * (rowS - 1) + 1] = cimag(s1);
                    S_idx[rowS - 1] = j + 1;
                }
                rowS++;
            }
            if (r12 || l_eq || l_eq_ex) {
                if (fill) {
                    H_data[2 * (rowH - 1)] = creal(h);
                    H_data[2 * (rowH - 1) + 1] = cimag(h);
                    H_idx[rowH - 1] = j + 1;
                    if (H_scale) H_scale[rowH - 1] = scale;
                }
                rowH++;
            }
        }
        if (fill) {
            H_ptr[i - row_begin + 1] = rowH;
            S_ptr[i - row_begin + 1] = rowS;
        }
#undef RKT
    }
#undef SM
#undef HM
    free(ac.v);
    nnz_out[0] = rowH - 1;
    nnz_out[1] = rowS - 1;
}

/* ------------------------------------------------------------------------ */
/* One-body matrices (mat_els.f90:47-118, 294-346; potentials.f90:35-43;      */
/* CAP_tools.f90:23-33)                                                       */
/* ------------------------------------------------------------------------ */

/* gau_leg%init (quad_tools.f90:29-52): stdlib gauss_legendre with an interval. */
static void gl_interval(int64_t q, const double *x0, const double *w0, double a, double b,
                        double *x, double *w) {
    for (int64_t s = 0; s < q; ++s) {
        x[s] = 0.5 * (b - a) * x0[s] + 0.5 * (b + a);
        w[s] = 0.5 * (b - a) * w0[s];
    }
}

void or_setup_S(const double *knots, int64_t n_knots, int64_t k, int64_t k_GL, double *S) {
    int64_t n = n_knots - k, nb = n - 2, n_iv = n_knots - 2 * k + 1;
    const double *bp = knots + (k - 1);
    double x0[64], w0[64], x[64], w[64];
    or_gauss_legendre(k_GL, x0, w0);
    memset(S, 0, sizeof(double) * 2 * (size_t)nb * nb);
    for (int64_t jb = 1; jb <= nb; ++jb)
        for (int64_t ib = 1; ib <= nb; ++ib) {
            if (llabs(jb - ib) >= k) continue;
            for (int64_t ir = 1; ir <= n_iv; ++ir) {
                if (!(supp(ir, ib + 1, k) && supp(ir, jb + 1, k))) continue;
                gl_interval(k_GL, x0, w0, bp[ir - 1], bp[ir], x, w);
                double *dst = S + 2 * ((jb - 1) * nb + (ib - 1));
                for (int64_t s = 0; s < k_GL; ++s) {
                    double Bi = or_bvalue(knots, n, k, x[s], 0, ir, ib + 1);
                    double Bj = or_bvalue(knots, n, k, x[s], 0, ir, jb + 1);
                    dst[0] = dst[0] + w[s] * Bi * Bj;
                }
            }
        }
}

void or_setup_H1p(const double *knots, int64_t n_knots, int64_t k, int64_t k_GL, int64_t Z,
                  int64_t l, int64_t cap_order, double cap_r0, double cap_eta_re,
                  double cap_eta_im, double *H) {
    int64_t n = n_knots - k, nb = n - 2, n_iv = n_knots - 2 * k + 1;
    const double *bp = knots + (k - 1);
    double x0[64], w0[64], x[64], w[64];
    or_gauss_legendre(k_GL, x0, w0);
    double complex eta = cap_eta_re + I * cap_eta_im;
    double complex *Hc = (double complex *)H;
    memset(H, 0, sizeof(double) * 2 * (size_t)nb * nb);
    for (int64_t jb = 1; jb <= nb; ++jb)
        for (int64_t ib = 1; ib <= nb; ++ib) {
            if (llabs(jb - ib) >= k) continue;
            for (int64_t ir = 1; ir <= n_iv; ++ir) {
                if (!(supp(ir, ib + 1, k) && supp(ir, jb + 1, k))) continue;
                gl_interval(k_GL, x0, w0, bp[ir - 1], bp[ir], x, w);
                double complex *dst = Hc + (jb - 1) * nb + (ib - 1);
                for (int64_t s = 0; s < k_GL; ++s) {
                    double r = x[s];
                    double Bi = or_bvalue(knots, n, k, r, 0, ir, ib + 1);
                    double Bj = or_bvalue(knots, n, k, r, 0, ir, jb + 1);
                    double DBj = or_bvalue(knots, n, k, r, 2, ir, jb + 1);
                    double V = 0.5 * (double)l * (double)(l + 1) / powi(r, 2) - (double)Z / r;
                    double complex cap = 0.0;
                    if (r >= cap_r0) cap = (-I) * eta * powi(r - cap_r0, cap_order);
                    *dst = *dst + w[s] * (-0.5 * Bi * DBj + (V + cap) * Bi * Bj);
                }
            }
        }
}

/* ------------------------------------------------------------------------ */
/* Dipole blocks (mat_els.f90:120-170, 348-390, 717-829; dipole.f90:8-146)    */
/* ------------------------------------------------------------------------ */

void or_setup_radial_dip(const double *knots, int64_t n_knots, int64_t k, int64_t k_GL,
                         int64_t gauge, double *r_mat, double *dr_mat, double *r_inv_mat) {
    int64_t n = n_knots - k, nb = n - 2, n_iv = n_knots - 2 * k + 1;
    const double *bp = knots + (k - 1);
    double x0[64], w0[64], x[64], w[64];
    or_gauss_legendre(k_GL, x0, w0);
    double complex *R = (double complex *)r_mat, *D = (double complex *)dr_mat,
                   *Ri = (double complex *)r_inv_mat;
    if (R) memset(R, 0, sizeof(double complex) * (size_t)nb * nb);
    if (D) memset(D, 0, sizeof(double complex) * (size_t)nb * nb);
    if (Ri) memset(Ri, 0, sizeof(double complex) * (size_t)nb * nb);
    for (int64_t jb = 1; jb <= nb; ++jb)
        for (int64_t ib = 1; ib <= nb; ++ib) {
            if (llabs(jb - ib) >= k) continue;
            for (int64_t ir = 1; ir <= n_iv; ++ir) {
                if (!(supp(ir, ib + 1, k) && supp(ir, jb + 1, k))) continue;
                gl_interval(k_GL, x0, w0, bp[ir - 1], bp[ir], x, w);
                size_t o = (size_t)(jb - 1) * nb + (ib - 1);
                for (int64_t s = 0; s < k_GL; ++s) {
                    double Bi = or_bvalue(knots, n, k, x[s], 0, ir, ib + 1);
                    double Bj = or_bvalue(knots, n, k, x[s], 0, ir, jb + 1);
                    if (gauge == 0) {
                        /* compute_radial_dip_len (mat_els.f90:348-367) */
                        R[o] = R[o] + w[s] * x[s] * Bi * Bj;
                    } else {
                        /* compute_radial_dip_vel (mat_els.f90:369-390) */
                        double DBj = or_bvalue(knots, n, k, x[s], 1, ir, jb + 1);
                        D[o] = D[o] + (-I) * w[s] * Bi * DBj;
                        Ri[o] = Ri[o] + (-I) * w[s] * Bi * Bj / x[s];
                    }
                }
            }
        }
}

/* ang_dip_red (mat_els.f90:811-828) */
static double ang_dip_red(int64_t L1, int64_t L2, int64_t la, int64_t lb, int64_t lc, int64_t ld) {
    double res = 0.0;
    if (lb == ld) res = res + fabs(or_six_j(L1, 1, L2, lc, lb, la) * or_C_red_mat(1, la, lc));
    if (la == lc) res = res + fabs(or_six_j(L1, 1, L2, ld, la, lb) * or_C_red_mat(1, lb, ld));
    return res;
}

/* dip_red_1p_len / dip_red_1p_vel (mat_els.f90:772-809) for (n, n_p, l, l_p) */
static double complex dip_red_1p(int64_t gauge, int64_t n, int64_t np, int64_t l, int64_t lp,
                                 int64_t nb, const double complex *R, const double complex *D,
                                 const double complex *Ri) {
    size_t o = (size_t)(np - 1) * nb + (n - 1);
    if (gauge == 0) return R[o] * or_C_red_mat(1, l, lp);
    if (llabs(l - lp) != 1) return 0.0;
    if (l > lp) return sqrt((double)l) * (D[o] - (double)(lp + 1) * Ri[o]);
    return -sqrt((double)lp) * (D[o] + (double)lp * Ri[o]);
}

/* dip_red_mat (mat_els.f90:739-770); confs(1) = (na,nb1; la,lb), confs(2) = (nc,nd; lc,ld) */
static double complex dip_red_mat(int64_t L1, int64_t L2, int64_t na, int64_t nb1, int64_t la,
                                  int64_t lb, int64_t nc, int64_t nd, int64_t lc, int64_t ld,
                                  int64_t gauge, int64_t nbas, const double complex *S,
                                  const double complex *R, const double complex *D,
                                  const double complex *Ri) {
    double complex r1 = 0.0, r2 = 0.0;
    double sq = sqrt((double)((2 * L1 + 1) * (2 * L2 + 1)));
    if (lb == ld) {
        double sg = ((la + lb + L2 + 1) & 1) ? -1.0 : 1.0;
        r1 = sg * sq * or_six_j(L1, 1, L2, lc, lb, la) *
             dip_red_1p(gauge, na, nc, la, lc, nbas, R, D, Ri) * S[(size_t)(nd - 1) * nbas + (nb1 - 1)];
    }
    if (la == lc) {
        double sg = ((la + ld + L1 + 1) & 1) ? -1.0 : 1.0;
        r2 = sg * sq * or_six_j(L1, 1, L2, ld, la, lb) *
             dip_red_1p(gauge, nb1, nd, lb, ld, nbas, R, D, Ri) * S[(size_t)(nc - 1) * nbas + (na - 1)];
    }
    return r1 + r2;
}

int64_t or_dip_block(const or_config *rows, int64_t n_rows, int64_t L1, int64_t M1, int64_t pi1,
                     const or_config *cols, int64_t n_cols, int64_t L2, int64_t M2, int64_t pi2,
                     int64_t q, int64_t compute, int64_t k, int64_t n_b, int64_t gauge,
                     const double *S, const double *r_mat, const double *dr_mat,
                     const double *r_inv_mat, int64_t *ptr, int64_t *idx, double *data) {
    const double complex *Sc = (const double complex *)S, *R = (const double complex *)r_mat,
                         *D = (const double complex *)dr_mat, *Ri = (const double complex *)r_inv_mat;
    int parity_allowed = (pi1 != 0) != (pi2 != 0);
    double ang = (((L1 - M1) & 1) ? -1.0 : 1.0) * or_three_j(L1, 1, L2, -M1, q, M2);
    if (fabs(ang) < 5e-16 || !parity_allowed || !compute) {
        if (ptr)
            for (int64_t i = 0; i <= n_rows; ++i) ptr[i] = 1;
        return 0;
    }
    int64_t p = 1;
    if (ptr) ptr[0] = 1;
    for (int64_t i = 0; i < n_rows; ++i) {
        int64_t na = rows[i].n1, nb1 = rows[i].n2, la = rows[i].l1, lb = rows[i].l2;
        for (int64_t j = 0; j < n_cols; ++j) {
            int64_t nc = cols[j].n1, nd = cols[j].n2, lc = cols[j].l1, ld = cols[j].l2;
            int support = llabs(na - nc) < k && llabs(nb1 - nd) < k;
            int support_ex = llabs(na - nd) < k && llabs(nb1 - nc) < k;
            int nz = 0;
            if (support) {
                if (ang_dip_red(L1, L2, la, lb, lc, ld) > 5e-16) nz = 1;
            } else if (support_ex) {
                if (ang_dip_red(L1, L2, la, lb, lc, ld) > 5e-16) nz = 1;
            }
            if (!nz) continue;
            if (idx) {
                /* dip_mat_neq (mat_els.f90:717-737) */
                double complex red = dip_red_mat(L1, L2, na, nb1, la, lb, nc, nd, lc, ld, gauge, n_b,
                                                 Sc, R, D, Ri);
                double complex red_ex = dip_red_mat(L1, L2, na, nb1, la, lb, nd, nc, ld, lc, gauge,
                                                    n_b, Sc, R, D, Ri);
                double sg = ((L2 + lc + ld) & 1) ? -1.0 : 1.0;
                double complex v = ang * (red + sg * red_ex);
                idx[p - 1] = j + 1;
                data[2 * (p - 1)] = creal(v);
                data[2 * (p - 1) + 1] = cimag(v);
            }
            p++;
        }
        if (ptr) ptr[i + 1] = p;
    }
    return p - 1;
}

/* ---- sparse_array_tools.f90:966-1074: CSR_mv, CSR_T_mv, CSR_mv_sym ------ */
void or_csr_mv(int64_t op, int64_t n_rows, int64_t n_cols, const int64_t *ptr,
               const int64_t *idx, const double *data, const double *x, double *y,
               double *scale) {
    const double complex *A = (const double complex *)data;
    const double complex *X = (const double complex *)x;
    double complex *Y = (double complex *)y;
    int64_t n_out = op == 1 ? n_cols : n_rows;
    for (int64_t i = 0; i < n_out; ++i) {
        Y[i] = 0.0;
        if (scale) scale[i] = 0.0;
    }
    if (op == 0) {
        /* y(i) = y(i) + A%data(j)*x(A%indices(j)), j ascending (:987-992) */
        for (int64_t i = 0; i < n_rows; ++i) {
            double complex acc = 0.0;
            for (int64_t j = ptr[i] - 1; j < ptr[i + 1] - 1; ++j) {
                acc = acc + A[j] * X[idx[j] - 1];
                if (scale) scale[i] += cabs(A[j]) * cabs(X[idx[j] - 1]);
            }
            Y[i] = acc;
        }
    } else if (op == 1) {
        /* y(A%indices(j)) = y(A%indices(j)) + A%data(j)*x(i) (:1022-1027) */
        for (int64_t i = 0; i < n_rows; ++i)
            for (int64_t j = ptr[i] - 1; j < ptr[i + 1] - 1; ++j) {
                Y[idx[j] - 1] += A[j] * X[i];
                if (scale) scale[idx[j] - 1] += cabs(A[j]) * cabs(X[i]);
            }
    } else {
        /* mkl_zcsrsymv('U') (:1053): the upper triangle (column >= row) of a
         * complex symmetric A; the commented loop of :1057-1072 spells it out
         * for upper-stored rows */
        for (int64_t i = 0; i < n_rows; ++i)
            for (int64_t j = ptr[i] - 1; j < ptr[i + 1] - 1; ++j) {
                int64_t c = idx[j] - 1;
                if (c < i) continue;
                Y[i] += A[j] * X[c];
                if (scale) scale[i] += cabs(A[j]) * cabs(X[c]);
                if (c > i) {
                    Y[c] += A[j] * X[i];
                    if (scale) scale[c] += cabs(A[j]) * cabs(X[i]);
                }
            }
    }
}

/* ---- block_tools.f90:188-234: CSR_from_block ---------------------------- */
int64_t or_csr_from_blocks(int64_t n_rb, int64_t n_cb, const int64_t *shapes, const int64_t *nnz,
                           const int64_t *const *ptr, const int64_t *const *idx,
                           const double *const *data, int64_t *out_ptr, int64_t *out_idx,
                           double *out_data) {
    int64_t p = 1, row = 0;
    for (int64_t i = 0; i < n_rb; ++i) {
        for (int64_t ri = 0; ri < shapes[2 * i]; ++ri) {
            int64_t col = 0;
            row += 1;
            out_ptr[row - 1] = p;
            for (int64_t j = 0; j < n_cb; ++j) {
                int64_t b = i + n_rb * j;
                if (nnz[b] > 0) { /* arrays_allocated() */
                    int64_t start = ptr[b][ri], end = ptr[b][ri + 1] - 1;
                    for (int64_t e = start; e <= end; ++e, ++p) {
                        out_idx[p - 1] = col + idx[b][e - 1];
                        out_data[2 * (p - 1)] = data[b][2 * (e - 1)];
                        out_data[2 * (p - 1) + 1] = data[b][2 * (e - 1) + 1];
                    }
                }
                col += shapes[2 * b + 1];
            }
        }
    }
    out_ptr[row] = p;
    return p - 1;
}
