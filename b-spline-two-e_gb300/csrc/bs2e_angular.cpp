// bs2e_angular.cpp -- exact Wigner 3j / 6j symbols and the LS angular weight.
//
// The reference obtains 3j/6j from GSL (src/tools/wigner_tools.f90:7-60) and
// combines them in ang_k_LS (:126-138) and C_red_mat (:107-112).  Here the
// Racah single sums are evaluated exactly: every term is scaled by a common
// integer denominator built from factorial ratios, so the sum is an exact
// big integer, and the symbol is sign * sqrt(NUM / DEN) of two big integers,
// rounded once to double.  Accidental zeros therefore come out as exact 0.0,
// which keeps the 5e-15 / 5e-16 pattern thresholds of hamiltonian.f90:174 and
// mat_els.f90:568 stable.
#include <cmath>
#include <cstdint>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "bs2e_internal.h"

namespace bs2e {
namespace {

// Non-negative big integer, 32-bit limbs, little-endian.
struct Big {
    std::vector<uint32_t> d;
    Big() {}
    explicit Big(uint64_t v) {
        while (v) {
            d.push_back((uint32_t)v);
            v >>= 32;
        }
    }
    bool zero() const { return d.empty(); }
    void trim() {
        while (!d.empty() && d.back() == 0) d.pop_back();
    }
    void mul_small(uint32_t m) {
        if (m == 0) {
            d.clear();
            return;
        }
        uint64_t carry = 0;
        for (auto &x : d) {
            uint64_t t = (uint64_t)x * m + carry;
            x = (uint32_t)t;
            carry = t >> 32;
        }
        if (carry) d.push_back((uint32_t)carry);
    }
    int bits() const {
        if (d.empty()) return 0;
        int b = 32 * (int)(d.size() - 1);
        uint32_t top = d.back();
        while (top) {
            b++;
            top >>= 1;
        }
        return b;
    }
};

Big mul(const Big &a, const Big &b) {
    Big r;
    if (a.zero() || b.zero()) return r;
    r.d.assign(a.d.size() + b.d.size(), 0);
    for (size_t i = 0; i < a.d.size(); ++i) {
        uint64_t carry = 0;
        for (size_t j = 0; j < b.d.size(); ++j) {
            uint64_t t = (uint64_t)a.d[i] * b.d[j] + r.d[i + j] + carry;
            r.d[i + j] = (uint32_t)t;
            carry = t >> 32;
        }
        size_t p = i + b.d.size();
        while (carry) {
            uint64_t t = (uint64_t)r.d[p] + carry;
            r.d[p] = (uint32_t)t;
            carry = t >> 32;
            ++p;
        }
    }
    r.trim();
    return r;
}

int cmp(const Big &a, const Big &b) {
    if (a.d.size() != b.d.size()) return a.d.size() < b.d.size() ? -1 : 1;
    for (size_t i = a.d.size(); i-- > 0;)
        if (a.d[i] != b.d[i]) return a.d[i] < b.d[i] ? -1 : 1;
    return 0;
}

Big add(const Big &a, const Big &b) {
    Big r;
    size_t n = std::max(a.d.size(), b.d.size());
    r.d.resize(n + 1, 0);
    uint64_t carry = 0;
    for (size_t i = 0; i < n; ++i) {
        uint64_t t = carry;
        if (i < a.d.size()) t += a.d[i];
        if (i < b.d.size()) t += b.d[i];
        r.d[i] = (uint32_t)t;
        carry = t >> 32;
    }
    r.d[n] = (uint32_t)carry;
    r.trim();
    return r;
}

// a - b for a >= b
Big sub(const Big &a, const Big &b) {
    Big r;
    r.d.resize(a.d.size(), 0);
    int64_t borrow = 0;
    for (size_t i = 0; i < a.d.size(); ++i) {
        int64_t t = (int64_t)a.d[i] - borrow - (i < b.d.size() ? (int64_t)b.d[i] : 0);
        borrow = t < 0;
        if (t < 0) t += ((int64_t)1 << 32);
        r.d[i] = (uint32_t)t;
    }
    r.trim();
    return r;
}

// Signed accumulator.
struct SBig {
    Big mag;
    bool neg = false;
    void add_signed(const Big &v, bool vneg) {
        if (v.zero()) return;
        if (mag.zero()) {
            mag = v;
            neg = vneg;
            return;
        }
        if (neg == vneg) {
            mag = add(mag, v);
            return;
        }
        int c = cmp(mag, v);
        if (c == 0) {
            mag = Big();
            neg = false;
        } else if (c > 0) {
            mag = sub(mag, v);
        } else {
            mag = sub(v, mag);
            neg = vneg;
        }
    }
};

// Top 62 bits of a as integer m with a ~= m * 2^e (exact when a < 2^62).
void top_bits(const Big &a, uint64_t &m, int &e) {
    int b = a.bits();
    if (b <= 62) {
        m = 0;
        for (size_t i = a.d.size(); i-- > 0;) m = (m << 32) | a.d[i];
        e = 0;
        return;
    }
    int shift = b - 62;
    m = 0;
    for (int bit = b - 1; bit >= shift; --bit) {
        uint32_t limb = a.d[bit / 32];
        m = (m << 1) | ((limb >> (bit % 32)) & 1u);
    }
    e = shift;
}

// sqrt(num / den), both positive.
double sqrt_ratio(const Big &num, const Big &den) {
    uint64_t mn, md;
    int en, ed;
    top_bits(num, mn, en);
    top_bits(den, md, ed);
    long double r = (long double)mn / (long double)md;
    int e = en - ed;
    // make the exponent even before the square root
    if (e & 1) {
        r *= 2.0L;
        e -= 1;
    }
    long double s = sqrtl(r);
    return (double)ldexpl(s, e / 2);
}

Big fact(int n) {
    Big r(1);
    for (int i = 2; i <= n; ++i) r.mul_small((uint32_t)i);
    return r;
}

// prod_{i=lo}^{hi} i (1 when hi < lo)
Big range_prod(int lo, int hi) {
    Big r(1);
    for (int i = std::max(lo, 1); i <= hi; ++i) r.mul_small((uint32_t)i);
    return r;
}

bool tri(int a, int b, int c) { return a >= 0 && b >= 0 && c >= 0 && c <= a + b && c >= std::abs(a - b); }

// Delta^2 as num/den: (a+b-c)!(a-b+c)!(-a+b+c)! / (a+b+c+1)!
void delta2(int a, int b, int c, Big &num, Big &den) {
    num = mul(num, mul(fact(a + b - c), mul(fact(a - b + c), fact(-a + b + c))));
    den = mul(den, fact(a + b + c + 1));
}

double three_j_exact(int j1, int j2, int j3, int m1, int m2, int m3) {
    if (m1 + m2 + m3 != 0) return 0.0;
    if (!tri(j1, j2, j3)) return 0.0;
    if (std::abs(m1) > j1 || std::abs(m2) > j2 || std::abs(m3) > j3) return 0.0;
    int al1 = j2 - j3 - m1, al2 = j1 - j3 + m2;          // t >= 0, al1, al2
    int be1 = j1 + j2 - j3, be2 = j1 - m1, be3 = j2 + m2;  // t <= be*
    int tmin = std::max(0, std::max(al1, al2));
    int tmax = std::min(be1, std::min(be2, be3));
    if (tmin > tmax) return 0.0;
    // Common denominator Dc = tmax!(tmax-al1)!(tmax-al2)!(be1-tmin)!(be2-tmin)!(be3-tmin)!
    SBig s;
    for (int t = tmin; t <= tmax; ++t) {
        Big term = range_prod(t + 1, tmax);
        term = mul(term, range_prod(t - al1 + 1, tmax - al1));
        term = mul(term, range_prod(t - al2 + 1, tmax - al2));
        term = mul(term, range_prod(be1 - t + 1, be1 - tmin));
        term = mul(term, range_prod(be2 - t + 1, be2 - tmin));
        term = mul(term, range_prod(be3 - t + 1, be3 - tmin));
        s.add_signed(term, (t & 1) != 0);
    }
    if (s.mag.zero()) return 0.0;
    Big Dc = mul(fact(tmax), mul(fact(tmax - al1), fact(tmax - al2)));
    Dc = mul(Dc, mul(fact(be1 - tmin), mul(fact(be2 - tmin), fact(be3 - tmin))));
    Big num(1), den(1);
    delta2(j1, j2, j3, num, den);
    num = mul(num, mul(fact(j1 + m1), fact(j1 - m1)));
    num = mul(num, mul(fact(j2 + m2), fact(j2 - m2)));
    num = mul(num, mul(fact(j3 + m3), fact(j3 - m3)));
    num = mul(num, mul(s.mag, s.mag));
    den = mul(den, mul(Dc, Dc));
    double v = sqrt_ratio(num, den);
    int ph = j1 - j2 - m3;
    bool neg = ((ph % 2) != 0) != s.neg;
    return neg ? -v : v;
}

double six_j_exact(int j1, int j2, int j3, int j4, int j5, int j6) {
    if (!tri(j1, j2, j3) || !tri(j1, j5, j6) || !tri(j4, j2, j6) || !tri(j4, j5, j3)) return 0.0;
    int a[4] = {j1 + j2 + j3, j1 + j5 + j6, j4 + j2 + j6, j4 + j5 + j3};
    int b[3] = {j1 + j2 + j4 + j5, j2 + j3 + j5 + j6, j3 + j1 + j6 + j4};
    int tmin = std::max(std::max(a[0], a[1]), std::max(a[2], a[3]));
    int tmax = std::min(b[0], std::min(b[1], b[2]));
    if (tmin > tmax) return 0.0;
    // Dc = prod_i (tmax-a_i)! prod_j (b_j-tmin)!
    SBig s;
    for (int t = tmin; t <= tmax; ++t) {
        Big term = fact(t + 1);
        for (int i = 0; i < 4; ++i) term = mul(term, range_prod(t - a[i] + 1, tmax - a[i]));
        for (int j = 0; j < 3; ++j) term = mul(term, range_prod(b[j] - t + 1, b[j] - tmin));
        s.add_signed(term, (t & 1) != 0);
    }
    if (s.mag.zero()) return 0.0;
    Big Dc(1);
    for (int i = 0; i < 4; ++i) Dc = mul(Dc, fact(tmax - a[i]));
    for (int j = 0; j < 3; ++j) Dc = mul(Dc, fact(b[j] - tmin));
    Big num(1), den(1);
    delta2(j1, j2, j3, num, den);
    delta2(j1, j5, j6, num, den);
    delta2(j4, j2, j6, num, den);
    delta2(j4, j5, j3, num, den);
    num = mul(num, mul(s.mag, s.mag));
    den = mul(den, mul(Dc, Dc));
    double v = sqrt_ratio(num, den);
    return s.neg ? -v : v;
}

std::mutex g_memo_mu;
std::map<std::tuple<int, int, int, int, int, int>, double> g_3j, g_6j, g_ang;

}  // namespace

double three_j(int ja, int jb, int jc, int ma, int mb, int mc) {
    auto key = std::make_tuple(ja, jb, jc, ma, mb, mc);
    {
        std::lock_guard<std::mutex> lk(g_memo_mu);
        auto it = g_3j.find(key);
        if (it != g_3j.end()) return it->second;
    }
    double v = three_j_exact(ja, jb, jc, ma, mb, mc);
    std::lock_guard<std::mutex> lk(g_memo_mu);
    g_3j[key] = v;
    return v;
}

double six_j(int ja, int jb, int jc, int jd, int je, int jf) {
    auto key = std::make_tuple(ja, jb, jc, jd, je, jf);
    {
        std::lock_guard<std::mutex> lk(g_memo_mu);
        auto it = g_6j.find(key);
        if (it != g_6j.end()) return it->second;
    }
    double v = six_j_exact(ja, jb, jc, jd, je, jf);
    std::lock_guard<std::mutex> lk(g_memo_mu);
    g_6j[key] = v;
    return v;
}

// C_red_mat (wigner_tools.f90:107-112)
static double c_red(int k, int a, int b) {
    double sg = (a & 1) ? -1.0 : 1.0;
    return sg * std::sqrt((double)((2 * a + 1) * (2 * b + 1))) * three_j(a, k, b, 0, 0, 0);
}

// ang_k_LS (wigner_tools.f90:126-138); confs(1) = (la, lb), confs(2) = (lc, ld)
double ang_k_LS(int k, int la, int lb, int lc, int ld, int L) {
    if (((la + k + lc) % 2) != 0 || ((lb + k + ld) % 2) != 0) return 0.0;
    double sg = ((lb + lc + L) & 1) ? -1.0 : 1.0;
    return sg * six_j(la, lb, L, ld, lc, k) * c_red(k, la, lc) * c_red(k, lb, ld);
}

}  // namespace bs2e

extern "C" {
BS2E_API double bs2e_ang_k_LS(int64_t k, int64_t la, int64_t lb, int64_t lc, int64_t ld,
                              int64_t L) {
    return bs2e::ang_k_LS((int)k, (int)la, (int)lb, (int)lc, (int)ld, (int)L);
}
BS2E_API double bs2e_three_j(int64_t ja, int64_t jb, int64_t jc, int64_t ma, int64_t mb,
                             int64_t mc) {
    return bs2e::three_j((int)ja, (int)jb, (int)jc, (int)ma, (int)mb, (int)mc);
}
BS2E_API double bs2e_six_j(int64_t ja, int64_t jb, int64_t jc, int64_t jd, int64_t je,
                           int64_t jf) {
    return bs2e::six_j((int)ja, (int)jb, (int)jc, (int)jd, (int)je, (int)jf);
}
}
