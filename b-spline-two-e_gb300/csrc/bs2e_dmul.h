// bs2e_dmul.h -- the product of two doubles with integer instructions only,
// rounded to nearest even exactly as the IEEE 754 multiply.
//
// GB300 runs FP64 at 1/64 of its FP32/integer issue rate (about two FP64
// operations per clock per SM), while an HBM-bound store of doubles needs a
// new element about every 0.37 clocks per SM.  The far-field R^k tiles are
// one product per stored element, so with the FP64 multiply the store is
// bound by the FP64 pipe; this form moves those products to the integer
// pipes and leaves the FP64 pipe to the near-field sums.  It returns x * y
// bit for bit (the store stays identical to the FP64 multiply) for positive
// normal x and y whose product is a normal double; other inputs take the
// FP64 multiply.
//
// Method: the 53-bit significands multiply to a 106-bit integer P in
// [2^104, 2^106); keeping its top 53 bits and rounding the dropped bits to
// nearest even gives the significand, and a carry out of the rounding moves
// into the exponent field because the result is assembled by integer
// addition of (exponent << 52) and the fraction.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define BS2E_HD __host__ __device__ __forceinline__
#else
#define BS2E_HD static inline
#endif

namespace bs2e {

BS2E_HD uint64_t dmul_umulhi(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

BS2E_HD uint64_t dbits(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    __builtin_memcpy(&u, &x, sizeof u);
    return u;
#endif
}

BS2E_HD double dfrom(uint64_t u) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double x;
    __builtin_memcpy(&x, &u, sizeof x);
    return x;
#endif
}

BS2E_HD double dmul_int(double x, double y) {
    const uint64_t bx = dbits(x), by = dbits(y);
    const int ex = (int)(bx >> 52), ey = (int)(by >> 52);  // sign bit 0 for the fast path
    // biased exponent of the result before normalisation
    const int e = ex + ey - 1023;
    if (ex == 0 || ey == 0 || ex >= 2047 || ey >= 2047 || e < 1 || e > 2045) return x * y;
    const uint64_t mx = (bx & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;
    const uint64_t my = (by & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;
    const uint64_t lo = mx * my, hi = dmul_umulhi(mx, my);  // P = hi 2^64 + lo
    const int top = (int)(hi >> 41);                        // bit 105 of P
    const int s = 52 + top;                                 // dropped bits
    const uint64_t mant = (hi << (64 - s)) | (lo >> s);     // 53 bits, leading bit set
    const uint64_t rem = lo & ((1ull << s) - 1), half = 1ull << (s - 1);
    const uint64_t up = (rem > half || (rem == half && (mant & 1))) ? 1ull : 0ull;
    return dfrom(((uint64_t)(e + top) << 52) + (mant - 0x0010000000000000ull) + up);
}

BS2E_HD uint32_t fbits(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    uint32_t u;
    __builtin_memcpy(&u, &x, sizeof u);
    return u;
#endif
}

BS2E_HD float ffrom(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float x;
    __builtin_memcpy(&x, &u, sizeof x);
    return x;
#endif
}

BS2E_HD float i2f_rn(int32_t r) {
#if defined(__CUDA_ARCH__)
    return __int2float_rn(r);
#else
    return (float)r;  // round to nearest even on IEEE hosts
#endif
}

// The FP32 pair (hi, lo) of x = v 2^s: hi = x rounded to float, lo = (x - hi)
// rounded to float, both to nearest even -- the values of
//   hi = (float)x;  lo = (float)(x - (double)hi);
// in FP64 arithmetic, formed with integer instructions for v >= 0 whose hi
// and lo are normal floats or zero (the others take those FP64 operations).
// hi keeps the top 24 of the 53 significand bits with the dropped 29 bits
// rounded; x - hi is that dropped part (an integer r, |r| <= 2^28, times the
// weight of the last significand bit), exact in FP64, so lo is r rounded to
// float with its exponent moved by integer addition.
BS2E_HD void split_scaled(double v, int s, float &hi, float &lo) {
    const uint64_t b = dbits(v);
    const int ev = (int)(b >> 52) - 1023 + s;  // exponent of x (sign bit 0 for v >= 0)
    if (b == 0) {
        hi = 0.0f;
        lo = 0.0f;
        return;
    }
    const int eb = (int)(b >> 52);
    if (eb == 0 || eb >= 2047 || ev + 127 < 1 || ev + 127 > 253) {
        const double x = v * dfrom((uint64_t)(1023 + s) << 52);
        hi = (float)x;
        lo = (float)(x - (double)hi);
        return;
    }
    const uint64_t m = (b & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;
    uint32_t mh = (uint32_t)(m >> 29);
    const uint32_t rem = (uint32_t)(m & ((1u << 29) - 1));
    const uint32_t up = (rem > (1u << 28) || (rem == (1u << 28) && (mh & 1u))) ? 1u : 0u;
    mh += up;
    int eh = ev;
    if (mh == (1u << 24)) {  // rounding carried into a new leading bit
        mh = 1u << 23;
        eh += 1;
    }
    hi = ffrom(((uint32_t)(eh + 127) << 23) | (mh & 0x007FFFFFu));
    const int32_t r = (int32_t)rem - (int32_t)(up << 29);
    if (r == 0) {
        lo = 0.0f;
        return;
    }
    // r 2^(ev - 52): r is exact in float up to 24 bits, rounded beyond
    const uint32_t fr = fbits(i2f_rn(r));
    const int ef = (int)((fr >> 23) & 0xFFu) + (ev - 52);
    if (ef < 1 || ef > 254) {
        const double x = v * dfrom((uint64_t)(1023 + s) << 52);
        lo = (float)(x - (double)hi);
        return;
    }
    lo = ffrom(fr + (uint32_t)((ev - 52) * (1 << 23)));
}

}  // namespace bs2e
