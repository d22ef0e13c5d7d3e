// bs2e_blockcsr.cu -- one CSR matrix from a block matrix of CSR blocks.
//
// Reference: CS_from_block / CSR_from_block and CS_from_block_diag /
// CSR_from_block_diag (src/tools/block_tools.f90:153-234, 289-348), which join
// the symmetry blocks of H and S and the dipole blocks D_q into the one CSR
// matrix the solvers use.  Row r of block row i is the concatenation, over
// block columns j, of row r of block (i, j) with its columns shifted by the
// column widths of blocks (i, 1..j-1); blocks with nnz = 0 contribute nothing
// but their width.
//
// Device: a count kernel (thread per output row) gives each row's length, the
// library's scan turns the lengths into the 1-based index_ptr, and a copy
// kernel (warp per output row) moves each segment with coalesced loads and
// stores.  Every block row pointer is checked against that block's nnz; a bad
// one sets the flag word and the row is skipped.
#include <cuda_runtime.h>

#include "bs2e_internal.h"

namespace bs2e {
namespace {

__device__ __forceinline__ int find_brow(const int64_t *row0, int n_rb, int64_t r) {
    int lo = 0, hi = n_rb - 1;  // largest i with row0[i] <= r
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (row0[mid] <= r)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__global__ void k_cat_count(CatArgs A, int64_t *__restrict__ cnt, int *__restrict__ bad) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= A.n_rows) return;
    const int i = find_brow(A.row0, A.n_rb, r);
    const int64_t ri = r - A.row0[i];
    int64_t c = 0;
    for (int j = 0; j < A.n_cb; ++j) {
        const CatBlock B = A.blocks[(size_t)i + (size_t)A.n_rb * j];
        if (B.nnz <= 0 || !B.ptr) continue;
        const int64_t j0 = B.ptr[ri] - 1, j1 = B.ptr[ri + 1] - 1;
        if (j0 < 0 || j1 < j0 || j1 > B.nnz) {
            atomicOr(bad, 1);
            continue;
        }
        c += j1 - j0;
    }
    cnt[r] = c;
}

__global__ void __launch_bounds__(256) k_cat_copy(CatArgs A, const int64_t *__restrict__ optr,
                                                  int64_t *__restrict__ oidx,
                                                  double2 *__restrict__ odat, int *__restrict__ bad) {
    const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= A.n_rows) return;  // warp-uniform
    const int i = find_brow(A.row0, A.n_rb, r);
    const int64_t ri = r - A.row0[i];
    int64_t o = optr[r] - 1;
    const int64_t o_end = optr[r + 1] - 1;
    for (int j = 0; j < A.n_cb; ++j) {
        const CatBlock B = A.blocks[(size_t)i + (size_t)A.n_rb * j];
        if (B.nnz <= 0 || !B.ptr) continue;
        const int64_t j0 = B.ptr[ri] - 1, j1 = B.ptr[ri + 1] - 1;
        if (j0 < 0 || j1 < j0 || j1 > B.nnz || o + (j1 - j0) > o_end) continue;  // counted as bad
        for (int64_t e = lane; e < j1 - j0; e += 32) {
            const int64_t c = B.idx[j0 + e];
            if (c < 1 || c > B.n_cols) atomicOr(bad, 2);
            oidx[o + e] = c + B.col0;
            odat[o + e] = B.data[j0 + e];
        }
        o += j1 - j0;
    }
}

}  // namespace

void launch_cat(bs2e_handle *h, const CatArgs &A, int64_t *cnt, int64_t *part, int64_t *optr,
                int64_t *oidx, double2 *odat, int *bad, bool copy) {
    if (A.n_rows <= 0) return;
    if (!copy) {
        k_cat_count<<<(unsigned)((A.n_rows + 255) / 256), 256, 0, h->stream>>>(A, cnt, bad);
        h->launches++;
        scan_one(h, cnt, A.n_rows, part, optr);
        return;
    }
    k_cat_copy<<<(unsigned)((A.n_rows * 32 + 255) / 256), 256, 0, h->stream>>>(A, optr, oidx, odat,
                                                                              bad);
    h->launches++;
}

}  // namespace bs2e
