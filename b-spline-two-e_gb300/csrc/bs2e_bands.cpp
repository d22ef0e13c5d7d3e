// bs2e_bands.cpp -- host-side planning of band work: bands that fit a buffer,
// their assignment to ranks, the rows of a band, and the join of band CSRs
// into a block CSR.  No CUDA: these run on any host thread or rank.
//
// The reference builds each symmetry block whole and joins blocks with
// CS_from_block_diag (src/tools/block_tools.f90:289-348); its OpenMP loop over
// symmetries (src/apps/main_basis_setup.f90:105-116) is the only
// parallelism.  Here a block is cut into n1 bands (rows of every channel
// with n1 in a range) so that blocks of 10^7 rows can be assembled piece by
// piece and spread over GPUs without any exchange between them.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/bs2e.h"

extern "C" {

BS2E_API bs2e_status bs2e_band_plan(int64_t n_blocks, const int64_t *n1_max,
                                    const int64_t *const *per_n1, int64_t max_bytes,
                                    int64_t n_ranks, int64_t cap, int64_t *bands,
                                    int64_t *n_bands) {
    if (n_blocks < 0 || n_ranks < 1 || max_bytes <= 0 || !n_bands || cap < 0 ||
        (n_blocks > 0 && (!n1_max || !per_n1)))
        return BS2E_ERR_ARG;
    struct Band {
        int64_t block, first, count, owner, bytes;
    };
    std::vector<Band> out;
    for (int64_t b = 0; b < n_blocks; ++b) {
        if (n1_max[b] < 0 || (n1_max[b] > 0 && !per_n1[b])) return BS2E_ERR_ARG;
        const int64_t *p = per_n1[b];
        int64_t a = 1;
        while (a <= n1_max[b]) {
            int64_t bytes = 0, e = a;
            while (e <= n1_max[b]) {
                const int64_t *t = p + 3 * (e - 1);
                if (t[0] < 0 || t[1] < 0 || t[2] < 0) return BS2E_ERR_ARG;
                const int64_t add = 24 * (t[1] + t[2]) + 16 * t[0];
                if (add + 16 > max_bytes) return BS2E_ERR_ARG;  // one n1 alone too large
                if (bytes + add + 16 > max_bytes) break;
                bytes += add;
                ++e;
            }
            if (bytes > 0) out.push_back(Band{b, a, e - a, 0, bytes + 16});
            a = e;
        }
    }
    *n_bands = (int64_t)out.size();
    if ((int64_t)out.size() > cap || (!bands && !out.empty())) return BS2E_ERR_ARG;
    // largest band first to the least loaded rank; ties by position / rank
    std::vector<int64_t> order(out.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int64_t)i;
    std::sort(order.begin(), order.end(), [&](int64_t x, int64_t y) {
        return out[x].bytes != out[y].bytes ? out[x].bytes > out[y].bytes : x < y;
    });
    std::vector<int64_t> load((size_t)n_ranks, 0);
    for (int64_t i : order) {
        int64_t r = 0;
        for (int64_t q = 1; q < n_ranks; ++q)
            if (load[q] < load[r]) r = q;
        out[i].owner = r;
        load[r] += out[i].bytes;
    }
    for (size_t i = 0; i < out.size(); ++i) {
        int64_t *d = bands + 5 * i;
        d[0] = out[i].block;
        d[1] = out[i].first;
        d[2] = out[i].count;
        d[3] = out[i].owner;
        d[4] = out[i].bytes;
    }
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_band_rows(const bs2e_config *configs, int64_t n_config,
                                    int64_t n1_first, int64_t n1_count, int64_t *rows,
                                    int64_t *n_rows) {
    if (n_config < 0 || n1_count < 0 || !n_rows || (n_config > 0 && !configs))
        return BS2E_ERR_ARG;
    int64_t m = 0;
    for (int64_t i = 0; i < n_config; ++i) {
        const int64_t n1 = configs[i].n1;
        if (n1 >= n1_first && n1 - n1_first < n1_count) {
            if (rows) rows[m] = i + 1;
            ++m;
        }
    }
    *n_rows = m;
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_band_merge(int64_t n_config, int64_t n_bands, const int64_t *n_rows,
                                     const int64_t *const *rows,
                                     const int64_t *const *index_ptr,
                                     const int64_t *const *indices, const double *const *data,
                                     int64_t *out_index_ptr, int64_t *out_indices,
                                     double *out_data) {
    if (n_config < 0 || n_bands < 0 || !out_index_ptr ||
        (n_bands > 0 && (!n_rows || !rows || !index_ptr || !indices || !data)))
        return BS2E_ERR_ARG;
    // source (band, local row) of every block row; each row exactly once
    std::vector<int64_t> src_band((size_t)n_config, -1), src_row((size_t)n_config, 0);
    for (int64_t b = 0; b < n_bands; ++b) {
        if (n_rows[b] < 0 || (n_rows[b] > 0 && (!rows[b] || !index_ptr[b]))) return BS2E_ERR_ARG;
        for (int64_t i = 0; i < n_rows[b]; ++i) {
            const int64_t r = rows[b][i] - 1;
            if (r < 0 || r >= n_config || src_band[(size_t)r] >= 0) return BS2E_ERR_ARG;
            src_band[(size_t)r] = b;
            src_row[(size_t)r] = i;
        }
    }
    int64_t pos = 0;
    out_index_ptr[0] = 1;
    for (int64_t r = 0; r < n_config; ++r) {
        const int64_t b = src_band[(size_t)r];
        if (b < 0) return BS2E_ERR_ARG;
        const int64_t i = src_row[(size_t)r];
        const int64_t s = index_ptr[b][i] - 1, e = index_ptr[b][i + 1] - 1;
        if (s < 0 || e < s) return BS2E_ERR_ARG;
        const int64_t len = e - s;
        if (len > 0) {
            if (!out_indices || !out_data || !indices[b] || !data[b]) return BS2E_ERR_ARG;
            std::memcpy(out_indices + pos, indices[b] + s, sizeof(int64_t) * (size_t)len);
            std::memcpy(out_data + 2 * pos, data[b] + 2 * s, 2 * sizeof(double) * (size_t)len);
        }
        pos += len;
        out_index_ptr[r + 1] = pos + 1;
    }
    return BS2E_OK;
}

}  // extern "C"
