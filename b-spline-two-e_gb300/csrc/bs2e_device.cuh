// bs2e_device.cuh -- device helpers shared by the CSR assembly kernels:
// enumeration of the (n_c, n_d) column runs of a row.
#pragma once
#include <cuda_runtime.h>

namespace bs2e {

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


}  // namespace bs2e
