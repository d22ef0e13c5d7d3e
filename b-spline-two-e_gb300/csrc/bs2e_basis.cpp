// bs2e_basis.cpp -- host-side planning: quadrature nodes, configuration lists
// and the per-block plan that the assembly kernels consume.
#include <cfloat>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "bs2e_internal.h"

namespace bs2e {

// Gauss-Legendre nodes and weights on [-1,1] (the reference takes them from
// fortran-lang/stdlib gauss_legendre, src/tools/quad_tools.f90:14-27).
// Newton's method on P_q from the asymptotic guess cos(pi (i-1/4)/(q+1/2)),
// carried out in long double and rounded once; nodes ascending.
void gauss_legendre(int q, double *x, double *w) {
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int i = 1; i <= q; ++i) {
        long double z = cosl(pi * ((long double)i - 0.25L) / ((long double)q + 0.5L));
        long double dp = 1.0L;
        for (int it = 0; it < 100; ++it) {
            long double p1 = 1.0L, p2 = 0.0L;
            for (int j = 1; j <= q; ++j) {
                long double p3 = p2;
                p2 = p1;
                p1 = ((2.0L * j - 1.0L) * z * p2 - (j - 1.0L) * p3) / j;
            }
            dp = (long double)q * (z * p1 - p2) / (z * z - 1.0L);
            long double dz = p1 / dp;
            z -= dz;
            if (fabsl(dz) <= 4.0L * LDBL_EPSILON * fabsl(z)) break;
        }
        // recompute the derivative at the converged node for the weight
        long double p1 = 1.0L, p2 = 0.0L;
        for (int j = 1; j <= q; ++j) {
            long double p3 = p2;
            p2 = p1;
            p1 = ((2.0L * j - 1.0L) * z * p2 - (j - 1.0L) * p3) / j;
        }
        dp = (long double)q * (z * p1 - p2) / (z * z - 1.0L);
        // i-th root counted from +1; store ascending
        x[q - i] = (double)z;
        w[q - i] = (double)(2.0L / ((1.0L - z * z) * dp * dp));
    }
    if (q % 2 == 1) x[q / 2] = 0.0;
}

// consistent() (src/tools/orbital_tools.f90:46-72) with a spin switch:
// singlet (the reference) drops equivalent configurations for odd L, the
// triplet drops them for even L.
static bool consistent(int64_t l1, int64_t l2, int64_t L, int64_t parity_odd, bool eqv,
                       int64_t spin) {
    if (eqv && ((spin == 0) ? (L % 2 != 0) : (L % 2 == 0))) return false;
    if (!(std::llabs(l1 - l2) <= L && L <= l1 + l2)) return false;
    bool par = ((l1 % 2) != 0) != ((l2 % 2) != 0);
    return par == (parity_odd != 0);
}

void plan_channels(BlockPlan &P, int K1) {
    const int nc = P.n_ch;
    const int64_t L = P.L;
    P.pairs.assign((size_t)nc * nc, PairInfo{});
    P.pair_k.assign((size_t)nc * nc * 2 * K1, 0);
    P.pair_a.assign((size_t)nc * nc * 2 * K1, 0.0);
    P.pair_af.assign((size_t)nc * nc * 2 * K1 * 2, 0.0f);
    const double exsign = P.spin ? -1.0 : 1.0;
    P.gated = false;
    for (int r = 0; r < nc; ++r)
        for (int c = 0; c < nc; ++c) {
            int la = P.ch_l1[r], lb = P.ch_l2[r], lc = P.ch_l1[c], ld = P.ch_l2[c];
            PairInfo &pi = P.pairs[(size_t)r * nc + c];
            double sgn = (((lc + ld + L) & 1) ? -1.0 : 1.0) * exsign;
            bool dir_ok = false, ex_ok = false;
            int nd = 0, nx = 0;
            size_t base = ((size_t)r * nc + c) * 2 * K1;
            for (int k = 0; k < K1; ++k) {
                double a = ang_k_LS(k, la, lb, lc, ld, (int)L);
                double ax = ang_k_LS(k, la, lb, ld, lc, (int)L);
                if (std::fabs(a) > 5e-15) dir_ok = true;
                if (std::fabs(ax) > 5e-15) ex_ok = true;
                if (!(std::fabs(a) < 5e-16)) {
                    P.pair_k[base + nd] = (int8_t)k;
                    P.pair_a[base + nd] = a;
                    nd++;
                }
                if (!(std::fabs(ax) < 5e-16)) {
                    P.pair_k[base + K1 + nx] = (int8_t)k;
                    P.pair_a[base + K1 + nx] = sgn * ax;
                    nx++;
                }
            }
            for (int t = 0; t < 2 * K1; ++t) {
                double a = P.pair_a[base + t];
                float hi = (float)a;
                float lo = (float)(a - (double)hi);
                P.pair_af[(base + t) * 2] = hi;
                P.pair_af[(base + t) * 2 + 1] = lo;
            }
            bool leq = (la == lc) && (lb == ld);
            bool leqx = (la == ld) && (lb == lc);
            // bit4: a listed weight lies in (5e-16, 5e-15] where no weight of that
            // term passes 5e-15, so whether the sums apply depends per entry on
            // the reference's r_12_allowed (the fill takes its gated path)
            const bool gated = (!dir_ok && nd > 0) || (!ex_ok && nx > 0);
            pi.flags = (dir_ok ? 1 : 0) | (ex_ok ? 2 : 0) | (leq ? 4 : 0) | (leqx ? 8 : 0) |
                       (gated ? 16 : 0);
            P.gated = P.gated || gated;
            pi.nd = nd;
            pi.nx = nx;
            pi.sgn = sgn;
        }
}

}  // namespace bs2e

extern "C" {

// count_configs (src/tools/orbital_tools.f90:119-216).
BS2E_API bs2e_status bs2e_configs(int64_t L, int64_t parity_odd, int64_t max_l_1p, int64_t n_b,
                                  int64_t k, int64_t max_n_b, int64_t n_all_l, int64_t l2_max,
                                  int64_t spin, bs2e_config *out, int64_t *n_config) {
    if (!n_config || L < 0 || max_l_1p < 0 || n_b < 1 || k < 2) return BS2E_ERR_ARG;
    int64_t cnt = 0;
    for (int64_t i = 0; i <= max_l_1p; ++i)
        for (int64_t j = 0; j <= i; ++j) {
            int64_t ni0 = std::min(i + 1, k - 1), nj0 = std::min(j + 1, k - 1);
            for (int64_t ni = ni0; ni <= n_b; ++ni) {
                if (ni > n_all_l && j > l2_max) continue;
                int64_t nj1 = (j == i) ? std::min(ni, max_n_b) : std::min(n_b, max_n_b);
                for (int64_t nj = nj0; nj <= nj1; ++nj) {
                    bool eqv = (i == j) && (ni == nj);
                    if (!bs2e::consistent(i, j, L, parity_odd, eqv, spin)) continue;
                    if (out) out[cnt] = bs2e_config{ni, nj, i, j, eqv ? 1 : 0};
                    cnt++;
                }
            }
        }
    *n_config = cnt;
    return BS2E_OK;
}
}
