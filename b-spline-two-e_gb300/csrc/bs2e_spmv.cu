// bs2e_spmv.cu -- products of the assembled CSR blocks with complex vectors.
//
// Reference: CSR_mv, CSR_T_mv and CSR_mv_sym (src/tools/sparse_array_tools.f90:
// 966-1074), the mat-vecs the solvers apply to H and S (eig_tools.f90:327-373,
// propagator_CN.f90:201-203, quasi_calcs.f90:838-871).  CSR_mv_sym calls
// mkl_zcsrsymv('U'): A is complex symmetric (not Hermitian: the CAP makes H
// complex symmetric) and only the entries with column >= row are read.
//
// One warp per row: lanes stride the row's entries, so the int64 column and
// complex128 value loads of a warp are contiguous (256 B + 512 B per step), the
// x gathers hit L1/L2 (columns of a row sit in a few narrow windows), and a
// shuffle reduction gives y(row).  The transposed and symmetric products add
// the scattered part with FP64 atomics into a zeroed y.  Every row pointer and
// column index is range-checked against nnz / n_cols; a bad one sets the flag
// word and is skipped, so malformed input reads nothing out of bounds.
#include <cuda_runtime.h>

#include "bs2e_internal.h"

namespace bs2e {
namespace {

// acc += a x in complex FP64.  The imaginary part of most entries is zero
// (the two-electron and overlap terms are real; only the CAP one-body term is
// complex), and the FP64 pipe, not HBM, bounds this kernel: a warp whose
// entries are all real (tested on the bit pattern, an integer op, and voted
// across the warp so that no predicated FMAs are issued) runs two FMAs per
// entry instead of four.
__device__ __forceinline__ void cmac(double &re, double &im, double2 a, double2 x) {
    re = fma(a.x, x.x, re);
    im = fma(a.x, x.y, im);
    const bool cplx = (__double_as_longlong(a.y) << 1) != 0;  // +-0 count as real
    if (__any_sync(__activemask(), cplx)) {
        // a compiler barrier keeps this a branch: predicated FMAs would still
        // occupy the FP64 pipe
        asm volatile("" ::: "memory");
        re = fma(-a.y, x.y, re);
        im = fma(a.y, x.x, im);
    }
}

// OP 0: y = A x.  OP 1: y += A^T x (y zeroed).  OP 2: y += U x + (U - diag)^T x
// with U the column >= row part of A (y zeroed).
template <int OP>
__global__ void __launch_bounds__(256) k_csr_mv(int64_t n_rows, int64_t n_cols, int64_t nnz,
                                                const int64_t *__restrict__ ptr,
                                                const int64_t *__restrict__ idx,
                                                const double2 *__restrict__ A,
                                                const double2 *__restrict__ x,
                                                double2 *__restrict__ y, int *__restrict__ bad) {
    const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= n_rows) return;  // warp-uniform
    const int64_t j0 = ptr[row] - 1, j1 = ptr[row + 1] - 1;
    if (j0 < 0 || j1 < j0 || j1 > nnz) {
        if (lane == 0) atomicOr(bad, 1);
        return;
    }
    double re = 0.0, im = 0.0;
    const double2 xr = (OP != 0) ? x[row] : make_double2(0.0, 0.0);
    // one entry of the row: c = idx - 1, a = A
    auto entry = [&](int64_t cc, double2 a) {
        const int64_t c = cc - 1;
        if (c < 0 || c >= n_cols) {
            atomicOr(bad, 2);
            return;
        }
        if (OP == 1) {
            double tr = 0.0, ti = 0.0;
            cmac(tr, ti, a, xr);
            atomicAdd(&y[c].x, tr);
            atomicAdd(&y[c].y, ti);
            return;
        }
        if (OP == 2 && c < row) return;
        cmac(re, im, a, x[c]);
        if (OP == 2 && c > row) {
            double tr = 0.0, ti = 0.0;
            cmac(tr, ti, a, xr);
            atomicAdd(&y[c].x, tr);
            atomicAdd(&y[c].y, ti);
        }
    };
    // two consecutive entries per lane and step: the column pair is one
    // 16-byte load, so a warp moves 512 B of columns and 1 KiB of values per
    // step with three load instructions.  idx is 8-byte aligned (checked on
    // the host); a leading entry at an address that is not 16-byte aligned
    // is taken first
    int64_t jb = j0;
    if ((reinterpret_cast<uintptr_t>(idx + jb) & 15) && jb < j1) {
        if (lane == 0) entry(idx[jb], A[jb]);
        ++jb;
    }
#pragma unroll 4
    for (int64_t j = jb + 2 * lane; j < j1; j += 64) {
        if (j + 1 < j1) {
            const longlong2 cc = *reinterpret_cast<const longlong2 *>(idx + j);
            const double2 a0 = A[j], a1 = A[j + 1];
            entry(cc.x, a0);
            entry(cc.y, a1);
        } else {
            entry(idx[j], A[j]);
        }
    }
    if (OP == 1) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if (lane == 0) {
        if (OP == 0) {
            y[row] = make_double2(re, im);
        } else {
            atomicAdd(&y[row].x, re);
            atomicAdd(&y[row].y, im);
        }
    }
}

// y = A x (op 0) with more loads in flight: each lane takes two consecutive
// entries per step as k_csr_mv does, but a batch of kMvSteps steps issues all
// its column-pair and value loads (streaming, evict-first: each is read once)
// before the x gathers, and the gathers before the FMAs.  One vote per batch
// decides whether the imaginary FMAs run (every entry of the batch then takes
// them right after its real ones; a real entry adds +-0, which leaves the
// sums unchanged), so each lane adds its entries' terms in the same order as
// k_csr_mv<0>.  Measured over the order-7 N=200 singlet H blocks (1.56e9
// entries, 37.4 GB per product): k_csr_mv<0> 10.95 ms (3.42 TB/s); batches of
// 2 steps 6.91 ms (5.42 TB/s, 58 registers), 3 steps 7.24 ms (76), 4 steps
// 8.24 ms (92: fewer resident warps).
constexpr int kMvSteps = 2;

__device__ __forceinline__ longlong2 ld_stream_ll2(const int64_t *p) {
    longlong2 v;
    asm volatile("ld.global.cs.v2.s64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(p));
    return v;
}

__device__ __forceinline__ double2 ld_stream_d2(const double2 *p) {
    double2 v;
    asm volatile("ld.global.cs.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "l"(p));
    return v;
}

// SYM: CSR_mv_sym with the same loads: entries below the diagonal are
// dropped, the row's sum is added to y (zeroed) atomically, and every entry
// above the diagonal adds a x(row) to y(column) as in k_csr_mv<2>.
template <bool SYM>
__global__ void __launch_bounds__(256) k_csr_mv_n(int64_t n_rows, int64_t n_cols, int64_t nnz,
                                                  const int64_t *__restrict__ ptr,
                                                  const int64_t *__restrict__ idx,
                                                  const double2 *__restrict__ A,
                                                  const double2 *__restrict__ x,
                                                  double2 *__restrict__ y,
                                                  int *__restrict__ bad) {
    const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= n_rows) return;  // warp-uniform
    const int64_t j0 = ptr[row] - 1, j1 = ptr[row + 1] - 1;
    if (j0 < 0 || j1 < j0 || j1 > nnz) {
        if (lane == 0) atomicOr(bad, 1);
        return;
    }
    double re = 0.0, im = 0.0;
    int64_t jb = j0;
    if ((reinterpret_cast<uintptr_t>(idx + jb) & 15) && jb < j1) {
        // a leading entry off the 16-byte boundary, as in k_csr_mv
        if (lane == 0) {
            const int64_t c = idx[jb] - 1;
            if (c < 0 || c >= n_cols) {
                atomicOr(bad, 2);
            } else if (!SYM || c >= row) {
                const double2 a = A[jb], xv = x[c];
                re = fma(a.x, xv.x, re);
                im = fma(a.x, xv.y, im);
                if ((__double_as_longlong(a.y) << 1) != 0) {
                    re = fma(-a.y, xv.y, re);
                    im = fma(a.y, xv.x, im);
                }
                if (SYM && c > row) {
                    const double2 xr = x[row];
                    double tr = fma(a.x, xr.x, 0.0), ti = fma(a.x, xr.y, 0.0);
                    tr = fma(-a.y, xr.y, tr);
                    ti = fma(a.y, xr.x, ti);
                    atomicAdd(&y[c].x, tr);
                    atomicAdd(&y[c].y, ti);
                }
            }
        }
        ++jb;
    }
    for (int64_t s = jb; s < j1; s += 64 * kMvSteps) {
        int64_t c[2 * kMvSteps];
        double2 a[2 * kMvSteps];
#pragma unroll
        for (int u = 0; u < kMvSteps; ++u) {
            const int64_t j = s + 64 * u + 2 * lane;
            if (j + 1 < j1) {
                const longlong2 cc = ld_stream_ll2(idx + j);
                c[2 * u] = cc.x;
                c[2 * u + 1] = cc.y;
                a[2 * u] = ld_stream_d2(A + j);
                a[2 * u + 1] = ld_stream_d2(A + j + 1);
            } else {
                c[2 * u] = j < j1 ? idx[j] : 0;  // 0: no entry here
                a[2 * u] = j < j1 ? A[j] : make_double2(0.0, 0.0);
                c[2 * u + 1] = 0;
                a[2 * u + 1] = make_double2(0.0, 0.0);
            }
        }
        double2 xv[2 * kMvSteps];
        bool cplx = false;
#pragma unroll
        for (int q = 0; q < 2 * kMvSteps; ++q) {
            const int64_t j = s + 64 * (q >> 1) + 2 * lane + (q & 1);
            const int64_t cq = c[q] - 1;
            xv[q] = make_double2(0.0, 0.0);
            if (j < j1) {
                if (cq < 0 || cq >= n_cols) {
                    atomicOr(bad, 2);
                    a[q] = make_double2(0.0, 0.0);
                } else if (SYM && cq < row) {
                    a[q] = make_double2(0.0, 0.0);  // below the diagonal: not read
                    c[q] = 0;
                } else {
                    xv[q] = __ldg(x + cq);
                }
            } else {
                c[q] = 0;
            }
            cplx |= (__double_as_longlong(a[q].y) << 1) != 0;
        }
        if (__any_sync(0xffffffffu, cplx)) {
            asm volatile("" ::: "memory");
#pragma unroll
            for (int q = 0; q < 2 * kMvSteps; ++q) {
                re = fma(a[q].x, xv[q].x, re);
                im = fma(a[q].x, xv[q].y, im);
                re = fma(-a[q].y, xv[q].y, re);
                im = fma(a[q].y, xv[q].x, im);
            }
        } else {
#pragma unroll
            for (int q = 0; q < 2 * kMvSteps; ++q) {
                re = fma(a[q].x, xv[q].x, re);
                im = fma(a[q].x, xv[q].y, im);
            }
        }
        if (SYM) {
            // the mirrored half: a x(row) into y(column) for columns past the row
            const double2 xr = x[row];
#pragma unroll
            for (int q = 0; q < 2 * kMvSteps; ++q) {
                const int64_t cq = c[q] - 1;
                if (cq > row && cq < n_cols) {
                    double tr = fma(a[q].x, xr.x, 0.0), ti = fma(a[q].x, xr.y, 0.0);
                    tr = fma(-a[q].y, xr.y, tr);
                    ti = fma(a[q].y, xr.x, ti);
                    atomicAdd(&y[cq].x, tr);
                    atomicAdd(&y[cq].y, ti);
                }
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if (lane == 0) {
        if (SYM) {
            atomicAdd(&y[row].x, re);
            atomicAdd(&y[row].y, im);
        } else {
            y[row] = make_double2(re, im);
        }
    }
}

}  // namespace

void launch_csr_mv(bs2e_handle *h, int op, int64_t n_rows, int64_t n_cols, int64_t nnz,
                   const int64_t *ptr, const int64_t *idx, const double2 *A, const double2 *x,
                   double2 *y, int *bad) {
    if (op != 0) {
        int64_t n_out = op == 1 ? n_cols : n_rows;
        cudaMemsetAsync(y, 0, sizeof(double2) * (size_t)n_out, h->stream);
    }
    if (n_rows == 0) return;
    const int threads = 256, rows_per_block = threads / 32;
    const int64_t blocks = (n_rows + rows_per_block - 1) / rows_per_block;
    if (op == 0)
        k_csr_mv_n<false><<<(unsigned)blocks, threads, 0, h->stream>>>(n_rows, n_cols, nnz, ptr,
                                                                       idx, A, x, y, bad);
    else if (op == 1)
        k_csr_mv<1><<<(unsigned)blocks, threads, 0, h->stream>>>(n_rows, n_cols, nnz, ptr, idx, A,
                                                                 x, y, bad);
    else
        k_csr_mv_n<true><<<(unsigned)blocks, threads, 0, h->stream>>>(n_rows, n_cols, nnz, ptr,
                                                                      idx, A, x, y, bad);
    h->launches++;
}

}  // namespace bs2e
