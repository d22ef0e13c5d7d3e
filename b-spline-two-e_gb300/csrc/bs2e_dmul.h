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

}  // namespace bs2e
