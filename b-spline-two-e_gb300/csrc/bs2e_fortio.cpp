// bs2e_fortio.cpp -- writer of the reference's block CSR files in gfortran's
// unformatted sequential format.
//
// Reference: CS_block_diag_store and CS_block_store
// (src/tools/block_tools.f90:386-415, 458-485), which write H_diag.dat,
// S_diag.dat and D_q.dat with plain unformatted WRITE statements:
//   'CSR' | block_shape(2) | shape(2) | per block: shape(2) | nnz |
//   [index_ptr(rows+1) | indices(nnz) | data(nnz)]   (arrays only when nnz > 0)
// with every integer int64 (-fdefault-integer-8) and data complex128.
//
// gfortran's record layout: each logical record is one or more subrecords of
// at most 2147483639 data bytes, each framed by 4-byte little-endian markers.
// The leading marker is +len for the last subrecord of a record and -len
// otherwise; the trailing marker is +len for the first subrecord and -len
// otherwise.  Records above 2 GiB (index and data arrays of large blocks)
// therefore span several subrecords.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "bs2e_internal.h"

namespace {

constexpr int64_t kMaxSub = 2147483639;

struct Writer {
    FILE *f = nullptr;
    int64_t max_sub = kMaxSub;
    bool ok = true;
    bool put(const void *p, size_t n) {
        if (ok && n && fwrite(p, 1, n, f) != n) ok = false;
        return ok;
    }
    bool marker(int64_t v) {
        int32_t m = (int32_t)v;
        return put(&m, 4);
    }
    // one logical record made of the concatenation of (ptr, bytes) pieces
    bool record(const std::vector<std::pair<const void *, int64_t>> &parts) {
        int64_t total = 0;
        for (auto &p : parts) total += p.second;
        int64_t done = 0;
        size_t pi = 0;
        int64_t poff = 0;
        bool first = true;
        do {
            int64_t len = total - done < max_sub ? total - done : max_sub;
            bool last = done + len == total;
            marker(last ? len : -len);
            int64_t left = len;
            while (left > 0) {
                int64_t take = parts[pi].second - poff < left ? parts[pi].second - poff : left;
                put((const char *)parts[pi].first + poff, (size_t)take);
                poff += take;
                left -= take;
                if (poff == parts[pi].second) {
                    ++pi;
                    poff = 0;
                }
            }
            marker(first ? len : -len);
            first = false;
            done += len;
        } while (done < total);
        return ok;
    }
    bool rec(const void *p, int64_t n) { return record({{p, n}}); }
};

bool write_block(Writer &w, const int64_t *shape, int64_t nnz, const int64_t *ptr,
                 const int64_t *idx, const double *data) {
    w.rec(shape, 16);
    w.rec(&nnz, 8);
    if (nnz > 0) {
        w.rec(ptr, 8 * (shape[0] + 1));
        w.rec(idx, 8 * nnz);
        w.rec(data, 16 * nnz);
    }
    return w.ok;
}

}  // namespace

extern "C" {

BS2E_API bs2e_status bs2e_write_block_diag(const char *path, int64_t n_blocks,
                                           const int64_t *shapes, const int64_t *nnz,
                                           const int64_t *const *index_ptr,
                                           const int64_t *const *indices,
                                           const double *const *data, int64_t max_subrecord) {
    if (!path || n_blocks < 0 || (n_blocks > 0 && (!shapes || !nnz))) return BS2E_ERR_ARG;
    Writer w;
    if (max_subrecord > 0) w.max_sub = max_subrecord;
    w.f = fopen(path, "wb");
    if (!w.f) return BS2E_ERR_ARG;
    int64_t block_shape[2] = {n_blocks, n_blocks}, shape[2] = {0, 0};
    for (int64_t i = 0; i < n_blocks; ++i) {
        shape[0] += shapes[2 * i];
        shape[1] += shapes[2 * i + 1];
    }
    w.rec("CSR", 3);
    w.rec(block_shape, 16);
    w.rec(shape, 16);
    for (int64_t i = 0; i < n_blocks && w.ok; ++i) {
        if (nnz[i] > 0 && (!index_ptr || !indices || !data || !index_ptr[i] || !indices[i] || !data[i])) {
            fclose(w.f);
            return BS2E_ERR_ARG;
        }
        write_block(w, shapes + 2 * i, nnz[i], nnz[i] > 0 ? index_ptr[i] : nullptr,
                    nnz[i] > 0 ? indices[i] : nullptr, nnz[i] > 0 ? data[i] : nullptr);
    }
    bool ok = w.ok;
    ok = (fclose(w.f) == 0) && ok;
    return ok ? BS2E_OK : BS2E_ERR_ARG;
}

BS2E_API bs2e_status bs2e_write_block(const char *path, int64_t n_rows_b, int64_t n_cols_b,
                                      const int64_t *shapes, const int64_t *nnz,
                                      const int64_t *const *index_ptr,
                                      const int64_t *const *indices, const double *const *data,
                                      int64_t max_subrecord) {
    if (!path || n_rows_b < 0 || n_cols_b < 0 || !shapes || !nnz) return BS2E_ERR_ARG;
    Writer w;
    if (max_subrecord > 0) w.max_sub = max_subrecord;
    w.f = fopen(path, "wb");
    if (!w.f) return BS2E_ERR_ARG;
    // blocks are column-major: block (i, j) at i + n_rows_b * j
    int64_t block_shape[2] = {n_rows_b, n_cols_b}, shape[2] = {0, 0};
    for (int64_t i = 0; i < n_rows_b && i < n_cols_b; ++i) {
        shape[0] += shapes[2 * (i + n_rows_b * i)];
        shape[1] += shapes[2 * (i + n_rows_b * i) + 1];
    }
    w.rec("CSR", 3);
    w.rec(block_shape, 16);
    w.rec(shape, 16);
    for (int64_t j = 0; j < n_cols_b && w.ok; ++j)
        for (int64_t i = 0; i < n_rows_b && w.ok; ++i) {
            int64_t b = i + n_rows_b * j;
            if (nnz[b] > 0 && (!index_ptr || !indices || !data || !index_ptr[b] || !indices[b] || !data[b])) {
                fclose(w.f);
                return BS2E_ERR_ARG;
            }
            write_block(w, shapes + 2 * b, nnz[b], nnz[b] > 0 ? index_ptr[b] : nullptr,
                        nnz[b] > 0 ? indices[b] : nullptr, nnz[b] > 0 ? data[b] : nullptr);
        }
    bool ok = w.ok;
    ok = (fclose(w.f) == 0) && ok;
    return ok ? BS2E_OK : BS2E_ERR_ARG;
}
}
