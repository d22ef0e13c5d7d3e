// bs2e_capi.cu -- the extern "C" entry points declared in include/bs2e.h.
//
// Every entry point locks the handle, makes the handle's device current and
// runs its kernels on the handle's stream.  Kernels are launched only through
// the launchers of bs2e_radial.cu / bs2e_assembly.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "bs2e_internal.h"

namespace bs2e {
size_t moments_smem(const Radial &g);
size_t fill_smem(const Radial &g);
}  // namespace bs2e

using namespace bs2e;

namespace {

struct Guard {
    bs2e_handle *h;
    std::lock_guard<std::mutex> lk;
    explicit Guard(bs2e_handle *hh) : h(hh), lk(hh->mu) { cudaSetDevice(hh->device); }
};

bs2e_status fail(bs2e_handle *h, bs2e_status st, const std::string &msg) {
    if (h) h->err = msg;
    return st;
}

#define CU(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(h, e_ == cudaErrorMemoryAllocation ? BS2E_ERR_NOMEM : BS2E_ERR_CUDA,  \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                  \
    } while (0)

template <class T>
cudaError_t dalloc(T **p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    return cudaMalloc((void **)p, n * sizeof(T));
}

template <class T>
void dfree(T *&p) {
    if (p) cudaFree((void *)p);
    p = nullptr;
}

// Waits for the stream and turns a set device error word into BS2E_ERR_TIMEOUT.
bs2e_status sync_check(bs2e_handle *h, const char *what) {
    CU(cudaStreamSynchronize(h->stream));
    CU(cudaGetLastError());
    int e = 0;
    CU(cudaMemcpy(&e, h->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        cudaMemset(h->d_err, 0, sizeof(int));
        if (e == 2)
            return fail(h, BS2E_ERR_COUNT,
                        std::string(what) + ": a row outside the band's row list was skipped");
        return fail(h, BS2E_ERR_TIMEOUT, std::string(what) + ": a bounded device wait expired");
    }
    return BS2E_OK;
}

// Number of basis splines (0-based b in [0,N)) non-zero on interval iv.
int splines_on(const Radial &g, int iv) {
    int lo = std::max(iv - 1, 0), hi = std::min(iv + g.k - 2, g.N - 1);
    return hi >= lo ? hi - lo + 1 : 0;
}

void free_block(DevBlock &b) {
    dfree(b.cfg);
    dfree(b.cfg_new);
    dfree(b.marks);
    dfree(b.lmap);
    dfree(b.chl);
    dfree(b.seg);
    dfree(b.pairs);
    dfree(b.pair_k);
    dfree(b.pair_a);
    dfree(b.pair_af);
    dfree(b.cntH);
    dfree(b.cntS);
    dfree(b.scan_tmp);
    dfree(b.stats);
    dfree(b.pfxH);
    dfree(b.pfxS);
    b.pfx_cap = 0;
    b.pfx_valid = false;
    b.cfg_cap = b.cfg_new_cap = b.seg_cap = b.pair_cap = b.cntH_cap = b.cntS_cap = b.scan_cap = 0;
    b.nnzH = b.nnzS = -1;
    b.valid = false;
}

// Grows a device buffer to hold at least n elements (contents not kept).
template <class T>
cudaError_t grow(T **p, int64_t &cap, int64_t n) {
    if (n <= cap && *p) return cudaSuccess;
    dfree(*p);
    int64_t c = std::max<int64_t>(n, 1);
    cudaError_t e = dalloc(p, (size_t)c);
    cap = (e == cudaSuccess) ? c : 0;
    return e;
}

#define TRY(x)                              \
    do {                                    \
        bs2e_status s_ = (x);               \
        if (s_ != BS2E_OK) return s_;       \
    } while (0)

// Device pointers from the caller: int64 arrays need 8-byte, complex128
// arrays 16-byte alignment (the kernels use 16-byte vector accesses).
inline bool aligned(const void *p, size_t a) { return ((uintptr_t)p % a) == 0; }

// Uploads the configuration list and, unless it is the block counted last,
// plans it on the device (channels, segment tables, order checks) and counts
// its non-zeros with both the construct and the count_nnz predicates.
bs2e_status ensure_counted(bs2e_handle *h, const bs2e_config *cf, int64_t n_config, int64_t L,
                           int64_t spin, int64_t full) {
    if (!cf && n_config > 0) return fail(h, BS2E_ERR_ARG, "configs is NULL");
    if (L < 0 || (spin != 0 && spin != 1) || (full != 0 && full != 1))
        return fail(h, BS2E_ERR_ARG, "L, spin or full out of range");
    if (n_config > ((int64_t)1 << 31) - 2) return fail(h, BS2E_ERR_ARG, "n_config too large");
    const Radial &g = h->g;
    {
        DevBlock &C = h->blk;
        if (!C.stats) CU(dalloc(&C.stats, 8));
        CU(grow(&C.cfg_new, C.cfg_new_cap, n_config));
        if (n_config > 0)
            CU(cudaMemcpyAsync(C.cfg_new, cf, sizeof(bs2e_config) * n_config,
                               cudaMemcpyHostToDevice, h->stream));
    }
    unsigned long long st[8];
    // is X the uploaded list?  (identity, then a device compare of every record)
    auto same = [&](const DevBlock &X, bool &eq) -> bs2e_status {
        eq = false;
        if (!(X.valid && X.L == L && X.spin == spin && X.full == full && X.n == n_config))
            return BS2E_OK;
        DevBlock &C = h->blk;
        CU(cudaMemsetAsync(C.stats, 0, 8 * sizeof(unsigned long long), h->stream));
        launch_cfg_equal(h, C.cfg_new, X.cfg, n_config, C.stats);
        CU(cudaMemcpyAsync(st, C.stats, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
        TRY(sync_check(h, "block compare"));
        eq = st[6] == 0;
        return BS2E_OK;
    };
    bool eq = false;
    TRY(same(h->blk, eq));
    if (eq) return BS2E_OK;  // the block counted last
    for (size_t i = 0; i < h->parked.size(); ++i) {
        TRY(same(h->parked[i].first, eq));
        if (!eq) continue;
        // a block counted earlier: make it current, park the current one first
        auto e = std::move(h->parked[i]);
        h->parked.erase(h->parked.begin() + (ptrdiff_t)i);
        if (h->blk.valid) h->parked.insert(h->parked.begin(), {h->blk, h->plan});
        else free_block(h->blk);
        h->blk = e.first;
        h->plan = e.second;
        return BS2E_OK;
    }
    if (h->blk.valid && h->cache_max > 0) {
        // park the current block; the upload moves to a fresh one
        DevBlock nb;
        std::swap(nb.cfg_new, h->blk.cfg_new);
        std::swap(nb.cfg_new_cap, h->blk.cfg_new_cap);
        h->parked.insert(h->parked.begin(), {h->blk, h->plan});
        h->blk = nb;
        int64_t rows = 0;
        size_t keep = 0;
        for (; keep < h->parked.size(); ++keep) {
            rows += h->parked[keep].first.n;
            if (keep >= (size_t)h->cache_max || rows > kBlockCacheRows) break;
        }
        while (h->parked.size() > keep) {
            free_block(h->parked.back().first);
            h->parked.pop_back();
        }
    }
    DevBlock &B = h->blk;
    if (!B.stats) CU(dalloc(&B.stats, 8));
    if (!B.marks) CU(dalloc(&B.marks, kMaxCh + 1));
    if (!B.lmap) CU(dalloc(&B.lmap, (size_t)kMaxL * kMaxL));
    if (!B.chl) CU(dalloc(&B.chl, kMaxCh));
    CU(cudaMemsetAsync(B.stats, 0, 8 * sizeof(unsigned long long), h->stream));
    B.valid = false;
    B.pfx_valid = false;
    BlockPlan &P = h->plan;
    P = BlockPlan();
    P.n_config = n_config;
    P.L = L;
    P.spin = spin;
    P.full = full;
    // channels: starts found on the device, ordered on the host
    std::vector<int4> marks(kMaxCh + 1);
    launch_chan_marks(h, n_config);
    CU(cudaMemcpyAsync(st, B.stats, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
    CU(cudaMemcpyAsync(marks.data(), B.marks, sizeof(int4) * marks.size(), cudaMemcpyDeviceToHost,
                       h->stream));
    TRY(sync_check(h, "block plan"));
    if (st[0] & 1ull) return fail(h, BS2E_ERR_ARG, "a configuration has n or l out of range");
    if (st[5] > (unsigned long long)kMaxCh)
        return fail(h, BS2E_ERR_ARG, "more than 256 channel runs in one block");
    marks.resize((size_t)st[5]);
    std::sort(marks.begin(), marks.end(), [](const int4 &a, const int4 &b) { return a.x < b.x; });
    std::vector<int> lmap((size_t)kMaxL * kMaxL, -1), chl;
    for (const int4 &m : marks) {
        int &slot = lmap[(size_t)m.y * kMaxL + m.z];
        if (slot >= 0)
            return fail(h, BS2E_ERR_ORDER, "channel (" + std::to_string(m.y) + "," +
                                               std::to_string(m.z) +
                                               ") is not contiguous in the configuration list");
        slot = P.n_ch++;
        P.ch_l1.push_back(m.y);
        P.ch_l2.push_back(m.z);
        P.ch_start.push_back(m.x);
        chl.push_back((m.y << 8) | m.z);
    }
    plan_channels(P, g.K1);
    const int S = g.N + 2;
    const int64_t nseg = (int64_t)P.n_ch * S;
    CU(grow(&B.seg, B.seg_cap, 3 * nseg));
    const int64_t npair = (int64_t)P.n_ch * P.n_ch;
    if (npair * 2 * g.K1 > B.pair_cap || !B.pairs) {
        dfree(B.pairs);
        dfree(B.pair_k);
        dfree(B.pair_a);
        dfree(B.pair_af);
        int64_t c = std::max<int64_t>(npair, 1);
        CU(dalloc(&B.pairs, (size_t)c));
        CU(dalloc(&B.pair_k, (size_t)c * 2 * g.K1));
        CU(dalloc(&B.pair_a, (size_t)c * 2 * g.K1));
        CU(dalloc(&B.pair_af, (size_t)c * 2 * g.K1 * 2));
        B.pair_cap = c * 2 * g.K1;
    }
    auto up = [&](void *dst, const void *src, size_t bytes) {
        return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->stream)
                     : cudaSuccess;
    };
    CU(up(B.lmap, lmap.data(), sizeof(int) * lmap.size()));
    CU(up(B.chl, chl.data(), sizeof(int) * chl.size()));
    CU(up(B.pairs, P.pairs.data(), sizeof(PairInfo) * P.pairs.size()));
    CU(up(B.pair_k, P.pair_k.data(), P.pair_k.size()));
    CU(up(B.pair_a, P.pair_a.data(), sizeof(double) * P.pair_a.size()));
    CU(up(B.pair_af, P.pair_af.data(), sizeof(float) * P.pair_af.size()));
    CU(cudaMemsetAsync(B.seg, 0xff, sizeof(int) * nseg, h->stream));              // base = -1
    CU(cudaMemsetAsync(B.seg + nseg, 0x7f, sizeof(int) * nseg, h->stream));       // lo = big
    CU(cudaMemsetAsync(B.seg + 2 * nseg, 0x00, sizeof(int) * nseg, h->stream));   // hi = 0
    launch_plan_seg(h, n_config);
    CU(grow(&B.cntH, B.cntH_cap, n_config));
    CU(grow(&B.cntS, B.cntS_cap, n_config));
    CU(grow(&B.scan_tmp, B.scan_cap, (n_config + 4095) / 4096 + 4));
    launch_block_count(h);
    CU(cudaMemcpyAsync(st, B.stats, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
    TRY(sync_check(h, "block count"));
    if (st[0] & 2ull)
        return fail(h, BS2E_ERR_ORDER, "configurations are not in basis order (n1 ascending, "
                                       "n2 consecutive within each (channel, n1) group)");
    const int64_t th = (int64_t)st[3], ts = (int64_t)st[4];
    B.nnzH = th;
    B.nnzS = ts;
    if ((int64_t)st[1] != th || (int64_t)st[2] != ts) {
        char buf[256];
        snprintf(buf, sizeof buf,
                 "count_nnz contract broken for this block: construct gives nnz_H=%lld nnz_S=%lld, "
                 "count_nnz gives %lld %lld",
                 (long long)th, (long long)ts, (long long)st[1], (long long)st[2]);
        return fail(h, BS2E_ERR_COUNT, buf);
    }
    std::swap(B.cfg, B.cfg_new);
    std::swap(B.cfg_cap, B.cfg_new_cap);
    B.L = L;
    B.spin = spin;
    B.full = full;
    B.n = n_config;
    B.valid = true;
    return BS2E_OK;
}

// Builds the FP32-pair copies of the one-body bands and decides whether the
// mixed assembly may use them (S real and every magnitude in range).
bs2e_status finish_one_body(bs2e_handle *h) {
    const Radial &g = h->g;
    dfree(h->d_Hbf);
    dfree(h->d_Sbf);
    CU(dalloc(&h->d_Hbf, (size_t)h->n_l * g.N * g.W));
    CU(dalloc(&h->d_Sbf, (size_t)g.N * g.W));
    launch_band_split(h);
    unsigned long long r[4];
    CU(cudaMemcpyAsync(r, h->d_range, sizeof(r), cudaMemcpyDeviceToHost, h->stream));
    TRY(sync_check(h, "one-body split"));
    // FP32-pair one-body and overlap products need every value and every
    // product of two values (H S and S S) in [2^-100, 2^124]: then the pairs'
    // low words and the TwoProd error terms stay normal FP32
    double v[4];
    for (int i = 0; i < 4; ++i) memcpy(&v[i], &r[i], sizeof(double));
    const double lo = 0x1p-100, hi = 0x1p124;
    const bool h_any = r[1] != 0, s_any = r[3] != 0;
    bool ok = true;
    if (s_any) ok = ok && v[2] >= lo && v[3] <= 0x1p62 && v[2] * v[2] >= lo && v[3] * v[3] <= hi;
    if (h_any) ok = ok && v[0] >= lo && v[1] <= hi;
    if (h_any && s_any) ok = ok && v[0] * v[2] >= lo && v[1] * v[3] <= hi;
    h->ff_one_body = h->s_real && ok;
    return BS2E_OK;
}

// One-particle reduced dipole dip_red_1p_len / _vel (mat_els.f90:772-809) as
// (alpha, beta): length alpha M1 with M1 = r_mat, velocity alpha M1 + beta M2
// with M1 = dr_mat, M2 = r_inv_mat.
void red1p(int gauge, int l, int lp, double &al, double &be) {
    al = be = 0.0;
    if (gauge == 0) {
        double sg = (l & 1) ? -1.0 : 1.0;
        al = sg * std::sqrt((double)((2 * l + 1) * (2 * lp + 1))) * three_j(l, 1, lp, 0, 0, 0);
        return;
    }
    if (std::abs(l - lp) != 1) return;
    if (l > lp) {
        al = std::sqrt((double)l);
        be = -(double)(lp + 1) * std::sqrt((double)l);
    } else {
        al = -std::sqrt((double)lp);
        be = -(double)lp * std::sqrt((double)lp);
    }
}

double c_red1(int a, int b) {  // C_red_mat(1, a, b)
    double sg = (a & 1) ? -1.0 : 1.0;
    return sg * std::sqrt((double)((2 * a + 1) * (2 * b + 1))) * three_j(a, 1, b, 0, 0, 0);
}

// Channel-pair coefficients of a dipole block (dip_mat_neq / dip_red_mat,
// mat_els.f90:717-770; ang_dip_red :811-828).
DipPair dip_pair(int L1, int L2, double ang3j, int gauge, int la, int lb, int lc, int ld) {
    DipPair p{};
    double adr = 0.0;
    if (lb == ld) adr += std::fabs(six_j(L1, 1, L2, lc, lb, la) * c_red1(la, lc));
    if (la == lc) adr += std::fabs(six_j(L1, 1, L2, ld, la, lb) * c_red1(lb, ld));
    p.ok = adr > 5e-16;
    const double sq = std::sqrt((double)((2 * L1 + 1) * (2 * L2 + 1)));
    const double sgx = ((L2 + lc + ld) & 1) ? -1.0 : 1.0;
    double al, be, f;
    if (lb == ld) {  // res_1: (n_a, n_c) with S(n_b, n_d)
        f = (((la + lb + L2 + 1) & 1) ? -1.0 : 1.0) * sq * six_j(L1, 1, L2, lc, lb, la) * ang3j;
        red1p(gauge, la, lc, al, be);
        p.c[0] = f * al;
        p.c[1] = f * be;
    }
    if (la == lc) {  // res_2: (n_b, n_d) with S(n_a, n_c)
        f = (((la + ld + L1 + 1) & 1) ? -1.0 : 1.0) * sq * six_j(L1, 1, L2, ld, la, lb) * ang3j;
        red1p(gauge, lb, ld, al, be);
        p.c[2] = f * al;
        p.c[3] = f * be;
    }
    if (lb == lc) {  // exchange res_1: (n_a, n_d) with S(n_b, n_c)
        f = sgx * (((la + lb + L2 + 1) & 1) ? -1.0 : 1.0) * sq * six_j(L1, 1, L2, ld, lb, la) * ang3j;
        red1p(gauge, la, ld, al, be);
        p.c[4] = f * al;
        p.c[5] = f * be;
    }
    if (la == ld) {  // exchange res_2: (n_b, n_c) with S(n_a, n_d)
        f = sgx * (((la + lc + L1 + 1) & 1) ? -1.0 : 1.0) * sq * six_j(L1, 1, L2, lc, la, lb) * ang3j;
        red1p(gauge, lb, lc, al, be);
        p.c[6] = f * al;
        p.c[7] = f * be;
    }
    for (int t = 0; t < 4; ++t)
        if (p.c[2 * t] != 0.0 || p.c[2 * t + 1] != 0.0) p.tm |= 1 << t;
    return p;
}

// Channel runs of a configuration list found on the device, in row order.
bs2e_status dip_channels(bs2e_handle *h, const bs2e_config *d_cfg, int64_t n,
                         std::vector<int4> &marks) {
    CU(cudaMemsetAsync(h->d_dip_stats, 0, 8 * sizeof(unsigned long long), h->stream));
    launch_chan_marks_on(h, d_cfg, n, h->d_dip_marks, kMaxCh + 1, h->d_dip_stats);
    unsigned long long st[8];
    marks.assign(kMaxCh + 1, make_int4(0, 0, 0, 0));
    CU(cudaMemcpyAsync(st, h->d_dip_stats, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
    CU(cudaMemcpyAsync(marks.data(), h->d_dip_marks, sizeof(int4) * marks.size(),
                       cudaMemcpyDeviceToHost, h->stream));
    TRY(sync_check(h, "dipole plan"));
    if (st[0] & 1ull) return fail(h, BS2E_ERR_ARG, "a configuration has n or l out of range");
    if (st[5] > (unsigned long long)kMaxCh)
        return fail(h, BS2E_ERR_ARG, "more than 256 channel runs in one symmetry");
    marks.resize((size_t)st[5]);
    std::sort(marks.begin(), marks.end(), [](const int4 &a, const int4 &b) { return a.x < b.x; });
    return BS2E_OK;
}

// Uploads, plans and counts one dipole block.  empty = the reference's
// zero block (3j factor below 5e-16, parity not changing, or compute = 0).
bs2e_status dip_prepare(bs2e_handle *h, const bs2e_config *rows, int64_t n_rows, int64_t L1,
                        int64_t M1, int64_t pi1, const bs2e_config *cols, int64_t n_cols,
                        int64_t L2, int64_t M2, int64_t pi2, int64_t q, int64_t compute,
                        DipDev &D, bool &empty, int64_t &nnz) {
    if (n_rows < 0 || n_cols < 0 || (n_rows > 0 && !rows) || (n_cols > 0 && !cols) || q < -1 ||
        q > 1 || L1 < 0 || L2 < 0)
        return fail(h, BS2E_ERR_ARG, "invalid dipole block arguments");
    if (h->dip_gauge < 0) return fail(h, BS2E_ERR_STATE, "radial dipole matrices not set");
    if (!h->have_one_body) return fail(h, BS2E_ERR_STATE, "overlap S not set (bs2e_set_one_body)");
    const Radial &g = h->g;
    double ang3j = (((L1 - M1) & 1) ? -1.0 : 1.0) *
                   three_j((int)L1, 1, (int)L2, (int)-M1, (int)q, (int)M2);
    bool parity_allowed = (pi1 != 0) != (pi2 != 0);
    empty = std::fabs(ang3j) < 5e-16 || !parity_allowed || !compute || n_rows == 0 || n_cols == 0;
    nnz = 0;
    if (empty) return BS2E_OK;
    if (!h->d_dip_stats) CU(dalloc(&h->d_dip_stats, 8));
    if (!h->d_dip_marks) CU(dalloc(&h->d_dip_marks, kMaxCh + 1));
    if (!h->d_dip_lmap) CU(dalloc(&h->d_dip_lmap, (size_t)2 * kMaxL * kMaxL));
    CU(grow(&h->d_dip_rows, h->dip_rows_cap, n_rows));
    CU(grow(&h->d_dip_cols, h->dip_cols_cap, n_cols));
    CU(cudaMemcpyAsync(h->d_dip_rows, rows, sizeof(bs2e_config) * n_rows, cudaMemcpyHostToDevice,
                       h->stream));
    CU(cudaMemcpyAsync(h->d_dip_cols, cols, sizeof(bs2e_config) * n_cols, cudaMemcpyHostToDevice,
                       h->stream));
    std::vector<int4> rm, cm;
    TRY(dip_channels(h, h->d_dip_rows, n_rows, rm));
    TRY(dip_channels(h, h->d_dip_cols, n_cols, cm));
    std::vector<int> lmap((size_t)2 * kMaxL * kMaxL, -1);
    std::vector<int> rl1, rl2, cl1, cl2;
    for (const int4 &m : rm) {  // rows: a channel may appear in several runs
        int &slot = lmap[(size_t)m.y * kMaxL + m.z];
        if (slot < 0) {
            slot = (int)rl1.size();
            rl1.push_back(m.y);
            rl2.push_back(m.z);
        }
    }
    for (const int4 &m : cm) {  // columns: each channel one contiguous run
        int &slot = lmap[(size_t)kMaxL * kMaxL + (size_t)m.y * kMaxL + m.z];
        if (slot >= 0)
            return fail(h, BS2E_ERR_ORDER, "a column channel is not contiguous in the configuration list");
        slot = (int)cl1.size();
        cl1.push_back(m.y);
        cl2.push_back(m.z);
    }
    const int nr = (int)rl1.size(), nc = (int)cl1.size();
    std::vector<DipPair> pairs((size_t)nr * nc);
    for (int r = 0; r < nr; ++r)
        for (int c = 0; c < nc; ++c)
            pairs[(size_t)r * nc + c] = dip_pair((int)L1, (int)L2, ang3j, h->dip_gauge, rl1[r],
                                                 rl2[r], cl1[c], cl2[c]);
    CU(grow(&h->d_dip_pairs, h->dip_pairs_cap, (int64_t)pairs.size()));
    CU(cudaMemcpyAsync(h->d_dip_pairs, pairs.data(), sizeof(DipPair) * pairs.size(),
                       cudaMemcpyHostToDevice, h->stream));
    CU(cudaMemcpyAsync(h->d_dip_lmap, lmap.data(), sizeof(int) * lmap.size(),
                       cudaMemcpyHostToDevice, h->stream));
    const int S = g.N + 2;
    const int64_t nseg = (int64_t)nc * S;
    CU(grow(&h->d_dip_seg, h->dip_seg_cap, 3 * nseg));
    CU(cudaMemsetAsync(h->d_dip_seg, 0xff, sizeof(int) * nseg, h->stream));
    CU(cudaMemsetAsync(h->d_dip_seg + nseg, 0x7f, sizeof(int) * nseg, h->stream));
    CU(cudaMemsetAsync(h->d_dip_seg + 2 * nseg, 0x00, sizeof(int) * nseg, h->stream));
    CU(cudaMemsetAsync(h->d_dip_stats, 0, 8 * sizeof(unsigned long long), h->stream));
    launch_plan_seg_on(h, h->d_dip_cols, n_cols, h->d_dip_lmap + kMaxL * kMaxL, S, h->d_dip_seg,
                       h->d_dip_seg + nseg, h->d_dip_seg + 2 * nseg, h->d_dip_stats);
    D.rows = h->d_dip_rows;
    D.n_rows = n_rows;
    D.lmap_r = h->d_dip_lmap;
    D.seg = h->d_dip_seg;
    D.nseg = nseg;
    D.n_ch_r = nr;
    D.n_ch_c = nc;
    D.pairs = h->d_dip_pairs;
    D.stats = h->d_dip_stats;
    CU(grow(&h->d_dip_cnt, h->dip_cnt_cap, n_rows));
    launch_dip_count(h, D, h->d_dip_cnt);
    unsigned long long st[8];
    CU(cudaMemcpyAsync(st, h->d_dip_stats, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
    TRY(sync_check(h, "dipole count"));
    if (st[0] & 2ull)
        return fail(h, BS2E_ERR_ORDER, "column configurations are not in basis order");
    nnz = (int64_t)st[3];
    return BS2E_OK;
}

}  // namespace

extern "C" {

BS2E_API void bs2e_default_opts(bs2e_opts *o) {
    if (!o) return;
    memset(o, 0, sizeof(*o));
    o->precision = BS2E_PREC_FP64;
    o->device = 0;
}

BS2E_API bs2e_status bs2e_create(const double *knots, int64_t n_knots, int64_t k, int64_t k_GL,
                                 int64_t max_k, const bs2e_opts *opts, bs2e_handle **out) {
    if (!out || !knots) return BS2E_ERR_ARG;
    *out = nullptr;
    if (k < 2 || k > kMaxOrder || k_GL < 1 || k_GL > kMaxGL || max_k < 0 || max_k + 1 > kMaxK1)
        return BS2E_ERR_ARG;
    int64_t n = n_knots - k;
    if (n - 2 < 1 || n_knots - 2 * k + 1 < 1) return BS2E_ERR_ARG;
    for (int64_t i = 1; i < n_knots; ++i)
        if (!(knots[i] >= knots[i - 1])) return BS2E_ERR_ARG;
    // every breakpoint interval must have positive length
    for (int64_t iv = 0; iv < n_knots - 2 * k + 1; ++iv)
        if (!(knots[k + iv] > knots[k - 1 + iv])) return BS2E_ERR_ARG;
    bs2e_opts o;
    bs2e_default_opts(&o);
    if (opts) o = *opts;
    if (o.precision != BS2E_PREC_FP64 && o.precision != BS2E_PREC_MIXED) return BS2E_ERR_ARG;
    if (o.stage_bytes < 0) return BS2E_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return BS2E_ERR_NODEV;
    if (o.device < 0 || o.device >= ndev) return BS2E_ERR_ARG;
    bs2e_handle *h = new (std::nothrow) bs2e_handle();
    if (!h) return BS2E_ERR_NOMEM;
    h->device = (int)o.device;
    h->precision = (int)o.precision;
    if (o.stage_bytes > 0) h->stage_limit = std::max<int64_t>(o.stage_bytes, 4096);
    cudaSetDevice(h->device);
    Radial &g = h->g;
    g.k = (int)k;
    g.q = (int)k_GL;
    g.K1 = (int)max_k + 1;
    g.n_knots = (int)n_knots;
    g.n = (int)n;
    g.N = (int)n - 2;
    g.n_iv = (int)(n_knots - 2 * k + 1);
    g.W = 2 * g.k - 1;
    g.tile = ((int64_t)g.K1 * g.W * g.W + 1) / 2 * 2;
    h->knots.assign(knots, knots + n_knots);
    h->glx.resize(g.q);
    h->glw.resize(g.q);
    gauss_legendre(g.q, h->glx.data(), h->glw.data());
    h->rk_done.assign(g.K1, 0);
    bs2e_status st = BS2E_OK;
    auto bad = [&](cudaError_t e) {
        if (e != cudaSuccess && st == BS2E_OK)
            st = (e == cudaErrorMemoryAllocation) ? BS2E_ERR_NOMEM : BS2E_ERR_CUDA;
    };
    bad(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    // the allocation-free lookup's static array, reserved now rather than at
    // its first call (a caller may have filled HBM by then)
    bad(noalloc_prepare(h->device, true));
    size_t q = g.q, kk = g.k, niv = g.n_iv, K1 = g.K1;
    bad(dalloc(&h->d_knots, (size_t)n_knots));
    bad(dalloc(&h->d_glx, q));
    bad(dalloc(&h->d_glw, q));
    bad(dalloc(&h->d_tab_r, niv * q));
    bad(dalloc(&h->d_tab_B, niv * q * kk));
    bad(dalloc(&h->d_tab_D2, niv * q * kk));
    bad(dalloc(&h->d_tab_D1, niv * q * kk));
    bad(dalloc(&h->d_tab_ri, niv * q * q));
    bad(dalloc(&h->d_tab_Bi, niv * q * q * kk));
    bad(dalloc(&h->d_mom, niv * K1 * 2 * kk * kk));
    bad(dalloc(&h->d_dint, niv * K1 * kk * kk * kk * kk));
    bad(dalloc(&h->d_dsym, niv * K1 * kk * kk * kk * kk));
    bad(dalloc(&h->d_tot, (size_t)2 * K1 * g.N * g.W));
    bad(dalloc(&h->d_err, 1));
    bad(dalloc(&h->d_range, 4));
    if (st == BS2E_OK) {
        bad(cudaMemcpy(h->d_knots, knots, sizeof(double) * n_knots, cudaMemcpyHostToDevice));
        bad(cudaMemcpy(h->d_glx, h->glx.data(), sizeof(double) * q, cudaMemcpyHostToDevice));
        bad(cudaMemcpy(h->d_glw, h->glw.data(), sizeof(double) * q, cudaMemcpyHostToDevice));
        bad(cudaMemset(h->d_err, 0, sizeof(int)));
    }
    if (st == BS2E_OK && (moments_smem(g) > 200 * 1024 || fill_smem(g) > 200 * 1024))
        st = BS2E_ERR_ARG;
    if (st != BS2E_OK) {
        bs2e_destroy(h);
        return st;
    }
    *out = h;
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_destroy(bs2e_handle *h) {
    if (!h) return BS2E_OK;
    {
        std::lock_guard<std::mutex> lk(h->mu);
        cudaSetDevice(h->device);
        if (h->stream) cudaStreamSynchronize(h->stream);
        free_block(h->blk);
        for (auto &e : h->parked) free_block(e.first);
        h->parked.clear();
        dfree(h->d_knots);
        dfree(h->d_glx);
        dfree(h->d_glw);
        dfree(h->d_tab_r);
        dfree(h->d_tab_B);
        dfree(h->d_tab_D2);
        dfree(h->d_tab_D1);
        dfree(h->d_dM1);
        dfree(h->d_dM2);
        dfree(h->d_dip_rows);
        dfree(h->d_dip_cols);
        dfree(h->d_dip_lmap);
        dfree(h->d_dip_seg);
        dfree(h->d_dip_pairs);
        dfree(h->d_dip_marks);
        dfree(h->d_dip_stats);
        dfree(h->d_dip_cnt);
        dfree(h->d_dip_part);
        dfree(h->d_rptrH);
        dfree(h->d_rptrS);
        dfree(h->d_band);
        dfree(h->d_band_idx);
        dfree(h->d_band_val);
        dfree(h->d_bptr);
        dfree(h->d_stage[0]);
        dfree(h->d_stage[1]);
        if (h->copy_stream) cudaStreamSynchronize(h->copy_stream), cudaStreamDestroy(h->copy_stream);
        for (int b = 0; b < 2; ++b) {
            if (h->ev_filled[b]) cudaEventDestroy(h->ev_filled[b]);
            if (h->ev_copied[b]) cudaEventDestroy(h->ev_copied[b]);
        }
        dfree(h->d_mv_ptr);
        dfree(h->d_mv_idx);
        dfree(h->d_mv_A);
        dfree(h->d_mv_x);
        dfree(h->d_mv_y);
        dfree(h->d_mv_bad);
        dfree(h->d_tab_ri);
        dfree(h->d_tab_Bi);
        dfree(h->d_mom);
        dfree(h->d_dint);
        dfree(h->d_dsym);
        dfree(h->d_tot);
        dfree(h->d_R);
        dfree(h->d_Rf);
        dfree(h->d_Rexp);
        dfree(h->d_err);
        dfree(h->d_range);
        dfree(h->d_Hbf);
        dfree(h->d_Sbf);
        dfree(h->d_Hb);
        dfree(h->d_Sb);
        if (h->stream) cudaStreamDestroy(h->stream);
    }
    delete h;
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_last_error(const bs2e_handle *h, char *buf, int64_t len) {
    if (!h || !buf || len <= 0) return BS2E_ERR_ARG;
    size_t n = std::min((size_t)len - 1, h->err.size());
    memcpy(buf, h->err.data(), n);
    buf[n] = 0;
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_sizes(const bs2e_handle *h, int64_t *n_b, int64_t *n_iv, int64_t *nnz4,
                                int64_t *nnz6) {
    if (!h) return BS2E_ERR_ARG;
    const Radial &g = h->g;
    int64_t s4 = 0, s6 = 0;
    for (int iv = 0; iv < g.n_iv; ++iv) {
        int64_t c = splines_on(g, iv);
        s4 += c * c;
        s6 += c * c * c * c;
    }
    if (n_b) *n_b = g.N;
    if (n_iv) *n_iv = g.n_iv;
    if (nnz4) *nnz4 = s4;
    if (nnz6) *nnz6 = s6;
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_slater(bs2e_handle *h) {
    if (!h) return BS2E_ERR_ARG;
    Guard G(h);
    launch_tabulate(h);
    launch_moments(h);
    launch_totals(h);
    TRY(sync_check(h, "slater"));
    h->slater_done = true;
    std::fill(h->rk_done.begin(), h->rk_done.end(), 0);
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_get_primitives(bs2e_handle *h, double *r_k, double *r_m_k,
                                         int64_t *idx4, double *r_d_k, int64_t *idx6) {
    if (!h) return BS2E_ERR_ARG;
    Guard G(h);
    if (!h->slater_done) return fail(h, BS2E_ERR_STATE, "bs2e_slater has not run");
    const Radial &g = h->g;
    const int k = g.k, K1 = g.K1, N = g.N, k2 = k * k;
    int64_t nnz4 = 0, nnz6 = 0;
    bs2e_sizes(h, nullptr, nullptr, &nnz4, &nnz6);
    std::vector<double> mom((size_t)g.n_iv * K1 * 2 * k2);
    CU(cudaMemcpy(mom.data(), h->d_mom, mom.size() * sizeof(double), cudaMemcpyDeviceToHost));
    auto ivrange = [&](int a, int c, int &lo, int &hi) {  // 0-based basis -> 0-based intervals
        lo = std::max(std::max(a, c) - k + 2, 0);
        hi = std::min(std::min(a, c) + 1, g.n_iv - 1);
    };
    if (r_k || r_m_k || idx4) {
        int64_t p = 0;
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) {
                if (std::abs(i - j) >= k) continue;
                int lo, hi;
                ivrange(i, j, lo, hi);
                for (int iv = lo; iv <= hi; ++iv, ++p) {
                    int si = i + 1 - iv, sj = j + 1 - iv;
                    for (int kk = 0; kk < K1; ++kk) {
                        const double *m = mom.data() + ((size_t)iv * K1 + kk) * 2 * k2;
                        if (r_k) r_k[p + nnz4 * kk] = m[si * k + sj];
                        if (r_m_k) r_m_k[p + nnz4 * kk] = m[k2 + si * k + sj];
                    }
                    if (idx4) {
                        idx4[3 * p] = iv + 1;
                        idx4[3 * p + 1] = i + 1;
                        idx4[3 * p + 2] = j + 1;
                    }
                }
            }
    }
    if (r_d_k || idx6) {
        std::vector<double> dint((size_t)g.n_iv * K1 * k2 * k2);
        CU(cudaMemcpy(dint.data(), h->d_dint, dint.size() * sizeof(double), cudaMemcpyDeviceToHost));
        int64_t p = 0;
        for (int jp = 0; jp < N; ++jp)
            for (int j = std::max(0, jp - k + 1); j <= std::min(N - 1, jp + k - 1); ++j)
                for (int ip = 0; ip < N; ++ip)
                    for (int i = std::max(0, ip - k + 1); i <= std::min(N - 1, ip + k - 1); ++i) {
                        int lo1, hi1, lo2, hi2;
                        ivrange(i, ip, lo1, hi1);
                        ivrange(j, jp, lo2, hi2);
                        for (int iv = std::max(lo1, lo2); iv <= std::min(hi1, hi2); ++iv, ++p) {
                            int pp = (i + 1 - iv) * k + (ip + 1 - iv);
                            int qq = (j + 1 - iv) * k + (jp + 1 - iv);
                            if (r_d_k)
                                for (int kk = 0; kk < K1; ++kk)
                                    r_d_k[p + nnz6 * kk] =
                                        dint[(((size_t)iv * K1 + kk) * k2 + pp) * k2 + qq];
                            if (idx6) {
                                int64_t *e = idx6 + 5 * p;
                                e[0] = iv + 1;
                                e[1] = i + 1;
                                e[2] = ip + 1;
                                e[3] = j + 1;
                                e[4] = jp + 1;
                            }
                        }
                    }
    }
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_rk(bs2e_handle *h, int64_t k_first, int64_t k_count) {
    if (!h) return BS2E_ERR_ARG;
    Guard G(h);
    const Radial &g = h->g;
    if (!h->slater_done) return fail(h, BS2E_ERR_STATE, "bs2e_slater has not run");
    if (k_first < 0 || k_count < 1 || k_first + k_count > g.K1)
        return fail(h, BS2E_ERR_ARG, "multipole range out of bounds");
    if (h->precision == BS2E_PREC_MIXED) {
        if (!h->d_Rf) CU(dalloc(&h->d_Rf, (size_t)g.N * g.N * g.tile));
        if (!h->d_Rexp) CU(dalloc(&h->d_Rexp, (size_t)g.N * g.N * g.K1));
    } else if (!h->d_R) {
        CU(dalloc(&h->d_R, (size_t)g.N * g.N * g.tile));
    }
    launch_rk_fill(h, (int)k_first, (int)k_count);
    TRY(sync_check(h, "rk"));
    for (int64_t kk = k_first; kk < k_first + k_count; ++kk) h->rk_done[kk] = 1;
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_rk_get_batch(bs2e_handle *h, int64_t n, const int64_t *keys,
                                       double *vals) {
    if (!h || n < 0 || (n > 0 && (!keys || !vals))) return BS2E_ERR_ARG;
    Guard G(h);
    if (!h->d_R && !h->d_Rf) return fail(h, BS2E_ERR_STATE, "bs2e_rk has not run");
    if (n == 0) return BS2E_OK;
    int64_t *dk = nullptr;
    double *dv = nullptr;
    CU(dalloc(&dk, (size_t)4 * n));
    CU(dalloc(&dv, (size_t)n * h->g.K1));
    CU(cudaMemcpyAsync(dk, keys, sizeof(int64_t) * 4 * n, cudaMemcpyHostToDevice, h->stream));
    launch_rk_gather(h, n, dk, dv);
    CU(cudaMemcpyAsync(vals, dv, sizeof(double) * n * h->g.K1, cudaMemcpyDeviceToHost, h->stream));
    bs2e_status st = sync_check(h, "rk_get");
    cudaFree(dk);
    cudaFree(dv);
    return st;
}

BS2E_API bs2e_status bs2e_rk_export(bs2e_handle *h, int64_t k, double *out, int64_t on_device) {
    if (!h || !out) return BS2E_ERR_ARG;
    Guard G(h);
    const Radial &g = h->g;
    if (k < 0 || k >= g.K1) return fail(h, BS2E_ERR_ARG, "rk_export: multipole out of range");
    if (!h->rk_done[k]) return fail(h, BS2E_ERR_STATE, "rk_export: multipole not built by bs2e_rk");
    const size_t n = (size_t)g.N * g.N * g.W * g.W;
    double *d = out;
    if (on_device && !aligned(out, 8)) return fail(h, BS2E_ERR_ARG, "rk_export: out needs 8-byte alignment");
    if (!on_device) CU(dalloc(&d, n));
    launch_rk_slice(h, (int)k, d);
    bs2e_status st = BS2E_OK;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && !on_device)
        e = cudaMemcpyAsync(out, d, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e != cudaSuccess) st = fail(h, BS2E_ERR_CUDA, cudaGetErrorString(e));
    bs2e_status st2 = sync_check(h, "rk_export");
    if (!on_device) cudaFree(d);
    return st != BS2E_OK ? st : st2;
}

BS2E_API bs2e_status bs2e_rk_get(bs2e_handle *h, const int64_t key[4], double *vals) {
    return bs2e_rk_get_batch(h, 1, key, vals);
}

BS2E_API bs2e_status bs2e_set_one_body(bs2e_handle *h, const double *H1p, int64_t n_l,
                                       const double *S) {
    if (!h || !H1p || !S || n_l < 1 || n_l > 32) return BS2E_ERR_ARG;
    Guard G(h);
    const Radial &g = h->g;
    const int N = g.N, W = g.W, k = g.k;
    std::vector<double2> Hb((size_t)n_l * N * W), Sb((size_t)N * W);
    bool sreal = true;
    for (int x = 0; x < N; ++x)
        for (int d = 0; d < W; ++d) {
            int y = x + d - (k - 1);
            double2 sv = make_double2(0.0, 0.0);
            if (y >= 0 && y < N) {
                size_t o = ((size_t)y * N + x) * 2;  // column-major (x, y)
                sv = make_double2(S[o], S[o + 1]);
                if (S[o + 1] != 0.0) sreal = false;
            }
            Sb[(size_t)x * W + d] = sv;
            for (int l = 0; l < n_l; ++l) {
                double2 hv = make_double2(0.0, 0.0);
                if (y >= 0 && y < N) {
                    size_t o = (((size_t)l * N + y) * N + x) * 2;
                    hv = make_double2(H1p[o], H1p[o + 1]);
                }
                Hb[((size_t)l * N + x) * W + d] = hv;
            }
        }
    dfree(h->d_Hb);
    dfree(h->d_Sb);
    CU(dalloc(&h->d_Hb, Hb.size()));
    CU(dalloc(&h->d_Sb, Sb.size()));
    CU(cudaMemcpy(h->d_Hb, Hb.data(), Hb.size() * sizeof(double2), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(h->d_Sb, Sb.data(), Sb.size() * sizeof(double2), cudaMemcpyHostToDevice));
    h->n_l = n_l;
    h->s_real = sreal;
    h->have_one_body = true;
    return finish_one_body(h);
}

BS2E_API bs2e_status bs2e_one_body(bs2e_handle *h, int64_t Z, int64_t n_l, int64_t cap_order,
                                   double cap_r0, double cap_eta_re, double cap_eta_im, double *H1p,
                                   double *S) {
    if (!h || n_l < 1 || n_l > 32 || cap_order < 0) return BS2E_ERR_ARG;
    Guard G(h);
    const Radial &g = h->g;
    if (!h->slater_done) return fail(h, BS2E_ERR_STATE, "bs2e_slater has not run (tabulation)");
    const int N = g.N, W = g.W, k = g.k;
    dfree(h->d_Hb);
    dfree(h->d_Sb);
    CU(dalloc(&h->d_Hb, (size_t)n_l * N * W));
    CU(dalloc(&h->d_Sb, (size_t)N * W));
    launch_one_body(h, Z, n_l, cap_order, cap_r0, cap_eta_re, cap_eta_im);
    TRY(sync_check(h, "one_body"));
    h->n_l = n_l;
    h->s_real = true;
    h->have_one_body = true;
    TRY(finish_one_body(h));
    if (H1p || S) {
        std::vector<double2> Hb((size_t)n_l * N * W), Sb((size_t)N * W);
        CU(cudaMemcpy(Hb.data(), h->d_Hb, Hb.size() * sizeof(double2), cudaMemcpyDeviceToHost));
        CU(cudaMemcpy(Sb.data(), h->d_Sb, Sb.size() * sizeof(double2), cudaMemcpyDeviceToHost));
        if (S) memset(S, 0, sizeof(double) * 2 * (size_t)N * N);
        if (H1p) memset(H1p, 0, sizeof(double) * 2 * (size_t)n_l * N * N);
        for (int x = 0; x < N; ++x)
            for (int d = 0; d < W; ++d) {
                int y = x + d - (k - 1);
                if (y < 0 || y >= N) continue;
                if (S) {
                    size_t o = ((size_t)y * N + x) * 2;
                    S[o] = Sb[(size_t)x * W + d].x;
                    S[o + 1] = Sb[(size_t)x * W + d].y;
                }
                if (H1p)
                    for (int l = 0; l < n_l; ++l) {
                        size_t o = (((size_t)l * N + y) * N + x) * 2;
                        H1p[o] = Hb[((size_t)l * N + x) * W + d].x;
                        H1p[o + 1] = Hb[((size_t)l * N + x) * W + d].y;
                    }
            }
    }
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_block_count_ex(bs2e_handle *h, const bs2e_config *configs,
                                         int64_t n_config, int64_t L, int64_t spin, int64_t full,
                                         int64_t *nnz_H, int64_t *nnz_S) {
    if (!h || !nnz_H || !nnz_S || n_config < 0) return BS2E_ERR_ARG;
    Guard G(h);
    TRY(ensure_counted(h, configs, n_config, L, spin, full));
    *nnz_H = h->blk.nnzH;
    *nnz_S = h->blk.nnzS;
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_block_count(bs2e_handle *h, const bs2e_config *configs,
                                      int64_t n_config, int64_t L, int64_t full, int64_t *nnz_H,
                                      int64_t *nnz_S) {
    return bs2e_block_count_ex(h, configs, n_config, L, 0, full, nnz_H, nnz_S);
}

// Checks shared by the fill entry points: every multipole built, one-body set
// and covering the block's l values, the block counted.
static bs2e_status fill_ready(bs2e_handle *h, const bs2e_config *configs, int64_t n_config, int64_t L,
                       int64_t spin, int64_t full) {
    for (int kk = 0; kk < h->g.K1; ++kk)
        if (!h->rk_done[kk]) return fail(h, BS2E_ERR_STATE, "bs2e_rk has not built every multipole");
    if (!h->have_one_body)
        return fail(h, BS2E_ERR_STATE, "one-body matrices not set (bs2e_set_one_body / bs2e_one_body)");
    TRY(ensure_counted(h, configs, n_config, L, spin, full));
    for (int c = 0; c < h->plan.n_ch; ++c)
        if (h->plan.ch_l1[c] >= h->n_l || h->plan.ch_l2[c] >= h->n_l)
            return fail(h, BS2E_ERR_ARG, "one-body matrices do not cover every l of the block");
    return BS2E_OK;
}

// The n_a (= n1) range of rows [r0, r1), and the fill mode: a range within
// one or two channels has about one row per tile; when the tile is large
// (staging it would leave an SM only a few CTAs, each with one busy warp) the
// range runs a warp per row.  Measured: order 9, 48.5 KB tiles, +20%; order
// 7, 15 KB tiles, staged tiles stay faster.
static void row_tiles(const bs2e_handle *h, const bs2e_config *cf, int64_t r0, int64_t r1,
                      FillRange &r) {
    int64_t a0 = INT64_MAX, a1 = 0;
    int runs = 0;
    for (int64_t i = r0; i < r1; ++i) {
        a0 = std::min<int64_t>(a0, cf[i].n1);
        a1 = std::max<int64_t>(a1, cf[i].n1);
        if (i == r0 || cf[i].l1 != cf[i - 1].l1 || cf[i].l2 != cf[i - 1].l2) ++runs;
    }
    r.a0 = (int)std::max<int64_t>(a0 == INT64_MAX ? 1 : a0, 1);
    r.a1 = (int)a1;
    r.rows_mode = runs <= 2 && h->g.tile * (int64_t)sizeof(double) > 32768;
}

// Range CSR pointers of rows [r0, r0 + n) into the handle's buffers.
static bs2e_status range_ptrs(bs2e_handle *h, int64_t r0, int64_t n) {
    if (n + 1 > h->rptr_cap) {
        dfree(h->d_rptrH);
        dfree(h->d_rptrS);
        h->rptr_cap = 0;
        CU(dalloc(&h->d_rptrH, (size_t)n + 1));
        CU(dalloc(&h->d_rptrS, (size_t)n + 1));
        h->rptr_cap = n + 1;
    }
    launch_block_scan(h, h->d_rptrH, h->d_rptrS, r0, n);
    return BS2E_OK;
}

// The copy stream and the two (filled, copied) event pairs of the staged
// host-output fills.
static bs2e_status ensure_copy_stream(bs2e_handle *h) {
    if (h->copy_stream) return BS2E_OK;
    CU(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
    for (int b = 0; b < 2; ++b) {
        CU(cudaEventCreateWithFlags(&h->ev_filled[b], cudaEventDisableTiming));
        CU(cudaEventCreateWithFlags(&h->ev_copied[b], cudaEventDisableTiming));
    }
    return BS2E_OK;
}

// Fills rows [r0, r0 + n) of the counted block into HOST arrays (range-local
// 1-based index_ptr): the range is cut into chunks that fit one of two
// staging areas in HBM; the fill of chunk c runs on the handle's stream while
// the copy stream moves chunk c - 1 to the host, so the device-to-host copy
// overlaps the assembly and device memory stays bounded.
static bs2e_status stream_fill(bs2e_handle *h, const bs2e_config *cf, int64_t r0, int64_t n,
                        int64_t *Hp, int64_t *Hi, double *Hd, int64_t *Sp, int64_t *Si,
                        double *Sd) {
    TRY(range_ptrs(h, r0, n));
    CU(cudaMemcpyAsync(Hp, h->d_rptrH, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, h->stream));
    CU(cudaMemcpyAsync(Sp, h->d_rptrS, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, h->stream));
    CU(cudaStreamSynchronize(h->stream));
    const int64_t nH = Hp[n] - 1, nS = Sp[n] - 1;
    if (nH == 0 && nS == 0) return sync_check(h, "block fill");
    TRY(ensure_copy_stream(h));
    // staging areas: the whole range if it fits, else the handle's limit
    // (8 GiB by default; a row holds at most 2 W^2 entries per column channel)
    const int64_t total = 24 * (nH + nS) + 64;
    const int64_t want = std::min<int64_t>(
        std::max<int64_t>(total, std::min<int64_t>((int64_t)64 << 20, h->stage_limit)),
        h->stage_limit);
    if (want > h->stage_cap) {
        CU(cudaStreamSynchronize(h->copy_stream));
        dfree(h->d_stage[0]);
        dfree(h->d_stage[1]);
        h->stage_cap = 0;
        CU(dalloc(&h->d_stage[0], (size_t)want));
        CU(dalloc(&h->d_stage[1], (size_t)want));
        h->stage_cap = want;
    }
    const int64_t cap = h->stage_cap - 64;
    // chunk boundaries: the most rows whose H + S entries fit one area
    std::vector<int64_t> cut{0};
    while (cut.back() < n) {
        const int64_t c0 = cut.back();
        if (24 * ((Hp[c0 + 1] - Hp[c0]) + (Sp[c0 + 1] - Sp[c0])) + 32 > cap)
            return fail(h, BS2E_ERR_NOMEM, "block fill: one row exceeds the staging area");
        int64_t c1 = c0 + 1, lo = c0 + 1, hi = n;
        while (lo <= hi) {
            int64_t mid = lo + (hi - lo) / 2;
            if (24 * ((Hp[mid] - Hp[c0]) + (Sp[mid] - Sp[c0])) + 32 <= cap) {
                c1 = mid;
                lo = mid + 1;
            } else {
                hi = mid - 1;
            }
        }
        cut.push_back(c1);
    }
    const int n_chunk = (int)cut.size() - 1;
    struct Lay {
        size_t oHd, oSi, oSd;
        int64_t hC, sC;
    };
    auto lay = [&](int c) {
        Lay L;
        L.hC = Hp[cut[c + 1]] - Hp[cut[c]];
        L.sC = Sp[cut[c + 1]] - Sp[cut[c]];
        L.oHd = (size_t)((8 * L.hC + 15) / 16 * 16);
        L.oSi = L.oHd + 16 * (size_t)L.hC;
        L.oSd = L.oSi + (size_t)((8 * L.sC + 15) / 16 * 16);
        return L;
    };
    cudaError_t e = cudaSuccess;
    // fill of chunk c into area c % 2, after the copies out of that area (chunk
    // c - 2) are done
    auto fill = [&](int c) {
        const int b = c & 1;
        const Lay L = lay(c);
        unsigned char *base = h->d_stage[b];
        if (e == cudaSuccess && c >= 2) e = cudaStreamWaitEvent(h->stream, h->ev_copied[b], 0);
        FillRange r;
        r.row0 = r0 + cut[c];
        r.row1 = r0 + cut[c + 1];
        r.ptr_row0 = r0;
        r.Hbase = Hp[cut[c]] - 1;
        r.Sbase = Sp[cut[c]] - 1;
        row_tiles(h, cf, r.row0, r.row1, r);
        if (e == cudaSuccess) {
            launch_block_fill(h, r, h->d_rptrH, h->d_rptrS, (int64_t *)base,
                              (double2 *)(base + L.oHd), (int64_t *)(base + L.oSi),
                              (double2 *)(base + L.oSd));
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaEventRecord(h->ev_filled[b], h->stream);
    };
    auto cp = [&](void *dst, const void *src, size_t bytes) {
        if (e == cudaSuccess && bytes)
            e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->copy_stream);
    };
    // the fill of chunk c + 1 is queued before the copies of chunk c are
    // issued: a copy to pageable memory may block the host until it is done
    fill(0);
    for (int c = 0; c < n_chunk && e == cudaSuccess; ++c) {
        if (c + 1 < n_chunk) fill(c + 1);
        const int b = c & 1;
        const Lay L = lay(c);
        const unsigned char *base = h->d_stage[b];
        if (e == cudaSuccess) e = cudaStreamWaitEvent(h->copy_stream, h->ev_filled[b], 0);
        cp(Hi + (Hp[cut[c]] - 1), base, 8 * (size_t)L.hC);
        cp(Hd + 2 * (Hp[cut[c]] - 1), base + L.oHd, 16 * (size_t)L.hC);
        cp(Si + (Sp[cut[c]] - 1), base + L.oSi, 8 * (size_t)L.sC);
        cp(Sd + 2 * (Sp[cut[c]] - 1), base + L.oSd, 16 * (size_t)L.sC);
        if (e == cudaSuccess) e = cudaEventRecord(h->ev_copied[b], h->copy_stream);
    }
    cudaError_t e2 = cudaStreamSynchronize(h->copy_stream);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) {
        cudaStreamSynchronize(h->stream);
        return fail(h, e == cudaErrorMemoryAllocation ? BS2E_ERR_NOMEM : BS2E_ERR_CUDA,
                    std::string("block fill (streamed): ") + cudaGetErrorString(e));
    }
    return sync_check(h, "block fill");
}

BS2E_API bs2e_status bs2e_block_fill_ex(bs2e_handle *h, const bs2e_config *configs,
                                        int64_t n_config, int64_t L, int64_t spin, int64_t full,
                                        int64_t *H_index_ptr, int64_t *H_indices, double *H_data,
                                        int64_t *S_index_ptr, int64_t *S_indices, double *S_data,
                                        int64_t out_on_device) {
    if (!h || n_config < 0) return BS2E_ERR_ARG;
    Guard G(h);
    TRY(fill_ready(h, configs, n_config, L, spin, full));
    const int64_t nH = h->blk.nnzH, nS = h->blk.nnzS;
    if (!H_index_ptr || !S_index_ptr || (nH > 0 && (!H_indices || !H_data)) ||
        (nS > 0 && (!S_indices || !S_data)))
        return fail(h, BS2E_ERR_ARG, "NULL output array");
    if (!out_on_device)
        return stream_fill(h, configs, 0, n_config, H_index_ptr, H_indices, H_data, S_index_ptr,
                           S_indices, S_data);
    if (!aligned(H_index_ptr, 8) || !aligned(S_index_ptr, 8) || !aligned(H_indices, 8) ||
        !aligned(S_indices, 8) || !aligned(H_data, 16) || !aligned(S_data, 16))
        return fail(h, BS2E_ERR_ARG, "device outputs: int64 arrays need 8-byte, data 16-byte alignment");
    launch_block_scan(h, H_index_ptr, S_index_ptr, 0, n_config);
    FillRange r;
    r.row0 = 0;
    r.row1 = n_config;
    r.a0 = 1;
    r.a1 = h->g.N;
    launch_block_fill(h, r, H_index_ptr, S_index_ptr, H_indices, (double2 *)H_data, S_indices,
                      (double2 *)S_data);
    CU(cudaGetLastError());
    return sync_check(h, "block fill");
}

// All symmetry blocks of a basis in one call: the loop of main_basis_setup.f90
// :105-116 over bas%syms as a batched count and a batched fill.  Each block
// goes through the single-block entry points (which take the handle's lock);
// the counts leave every block in the handle's block cache, so the fills that
// follow reuse their plans.  A failure names the block it happened in.
static bs2e_status blocks_args_ok(int64_t n_blocks, const bs2e_config *const *configs,
                                  const int64_t *n_config, const int64_t *L, const int64_t *spin) {
    if (n_blocks < 0) return BS2E_ERR_ARG;
    if (n_blocks > 0 && (!configs || !n_config || !L || !spin)) return BS2E_ERR_ARG;
    return BS2E_OK;
}

static void clear_error(bs2e_handle *h) {
    std::lock_guard<std::mutex> lk(h->mu);
    h->err.clear();
}

static bs2e_status block_failed(bs2e_handle *h, int64_t i, bs2e_status st) {
    std::lock_guard<std::mutex> lk(h->mu);
    h->err = "block " + std::to_string(i) + ": " +
             (h->err.empty() ? "invalid argument (status " + std::to_string(st) + ")" : h->err);
    return st;
}

BS2E_API bs2e_status bs2e_blocks_count_all(bs2e_handle *h, int64_t n_blocks,
                                           const bs2e_config *const *configs,
                                           const int64_t *n_config, const int64_t *L,
                                           const int64_t *spin, int64_t full, int64_t *nnz_H,
                                           int64_t *nnz_S) {
    if (!h || blocks_args_ok(n_blocks, configs, n_config, L, spin) != BS2E_OK ||
        (n_blocks > 0 && (!nnz_H || !nnz_S)))
        return BS2E_ERR_ARG;
    for (int64_t i = 0; i < n_blocks; ++i) {
        clear_error(h);
        const bs2e_status st = bs2e_block_count_ex(h, configs[i], n_config[i], L[i], spin[i], full,
                                                   &nnz_H[i], &nnz_S[i]);
        if (st != BS2E_OK) return block_failed(h, i, st);
    }
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_blocks_fill_all(bs2e_handle *h, int64_t n_blocks,
                                          const bs2e_config *const *configs,
                                          const int64_t *n_config, const int64_t *L,
                                          const int64_t *spin, int64_t full,
                                          int64_t *const *H_index_ptr, int64_t *const *H_indices,
                                          double *const *H_data, int64_t *const *S_index_ptr,
                                          int64_t *const *S_indices, double *const *S_data,
                                          int64_t out_on_device) {
    if (!h || blocks_args_ok(n_blocks, configs, n_config, L, spin) != BS2E_OK ||
        (n_blocks > 0 && (!H_index_ptr || !H_indices || !H_data || !S_index_ptr ||
                          !S_indices || !S_data)))
        return BS2E_ERR_ARG;
    for (int64_t i = 0; i < n_blocks; ++i) {
        clear_error(h);
        const bs2e_status st = bs2e_block_fill_ex(
            h, configs[i], n_config[i], L[i], spin[i], full, H_index_ptr[i], H_indices[i],
            H_data[i], S_index_ptr[i], S_indices[i], S_data[i], out_on_device);
        if (st != BS2E_OK) return block_failed(h, i, st);
    }
    return BS2E_OK;
}

// Rows [row_first, row_first + row_count) of a block.
static bs2e_status check_rows(bs2e_handle *h, int64_t n_config, int64_t row_first, int64_t row_count) {
    if (row_first < 0 || row_count < 0 || row_first + row_count > n_config)
        return fail(h, BS2E_ERR_ARG, "row range outside the block");
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_block_count_rows(bs2e_handle *h, const bs2e_config *configs,
                                           int64_t n_config, int64_t L, int64_t spin,
                                           int64_t full, int64_t row_first, int64_t row_count,
                                           int64_t *nnz_H, int64_t *nnz_S) {
    if (!h || n_config < 0 || !nnz_H || !nnz_S) return BS2E_ERR_ARG;
    Guard G(h);
    TRY(check_rows(h, n_config, row_first, row_count));
    TRY(ensure_counted(h, configs, n_config, L, spin, full));
    TRY(range_ptrs(h, row_first, row_count));
    int64_t eH = 1, eS = 1;
    CU(cudaMemcpyAsync(&eH, h->d_rptrH + row_count, 8, cudaMemcpyDeviceToHost, h->stream));
    CU(cudaMemcpyAsync(&eS, h->d_rptrS + row_count, 8, cudaMemcpyDeviceToHost, h->stream));
    TRY(sync_check(h, "block count (rows)"));
    *nnz_H = eH - 1;
    *nnz_S = eS - 1;
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_block_fill_rows(bs2e_handle *h, const bs2e_config *configs,
                                          int64_t n_config, int64_t L, int64_t spin, int64_t full,
                                          int64_t row_first, int64_t row_count,
                                          int64_t *H_index_ptr, int64_t *H_indices,
                                          double *H_data, int64_t *S_index_ptr,
                                          int64_t *S_indices, double *S_data,
                                          int64_t out_on_device) {
    if (!h || n_config < 0) return BS2E_ERR_ARG;
    Guard G(h);
    TRY(check_rows(h, n_config, row_first, row_count));
    TRY(fill_ready(h, configs, n_config, L, spin, full));
    if (!H_index_ptr || !S_index_ptr) return fail(h, BS2E_ERR_ARG, "NULL output array");
    if (!out_on_device)
        return stream_fill(h, configs, row_first, row_count, H_index_ptr, H_indices, H_data,
                           S_index_ptr, S_indices, S_data);
    if (!aligned(H_index_ptr, 8) || !aligned(S_index_ptr, 8) || !aligned(H_indices, 8) ||
        !aligned(S_indices, 8) || !aligned(H_data, 16) || !aligned(S_data, 16))
        return fail(h, BS2E_ERR_ARG, "device outputs: int64 arrays need 8-byte, data 16-byte alignment");
    launch_block_scan(h, H_index_ptr, S_index_ptr, row_first, row_count);
    FillRange r;
    r.row0 = row_first;
    r.row1 = row_first + row_count;
    r.ptr_row0 = row_first;
    row_tiles(h, configs, r.row0, r.row1, r);
    launch_block_fill(h, r, H_index_ptr, S_index_ptr, H_indices, (double2 *)H_data, S_indices,
                      (double2 *)S_data);
    CU(cudaGetLastError());
    return sync_check(h, "block fill (rows)");
}

// The two HBM staging areas of host-output fills, each at least `bytes`.
static bs2e_status ensure_stage(bs2e_handle *h, int64_t bytes) {
    if (bytes <= h->stage_cap && h->d_stage[0] && h->d_stage[1]) return BS2E_OK;
    if (h->copy_stream) CU(cudaStreamSynchronize(h->copy_stream));
    CU(cudaStreamSynchronize(h->stream));
    dfree(h->d_stage[0]);
    dfree(h->d_stage[1]);
    h->stage_cap = 0;
    const int64_t want = std::max<int64_t>(bytes, 256);
    CU(dalloc(&h->d_stage[0], (size_t)want));
    CU(dalloc(&h->d_stage[1], (size_t)want));
    h->stage_cap = want;
    return BS2E_OK;
}

// 1-based CSR pointers of the whole counted block (a scan of its row
// counts), built once per counted block for band fills.
static bs2e_status ensure_prefix(bs2e_handle *h) {
    DevBlock &B = h->blk;
    if (B.pfx_valid) return BS2E_OK;
    const int64_t n = h->plan.n_config;
    if (n + 1 > B.pfx_cap) {
        dfree(B.pfxH);
        dfree(B.pfxS);
        B.pfx_cap = 0;
        CU(dalloc(&B.pfxH, (size_t)n + 1));
        CU(dalloc(&B.pfxS, (size_t)n + 1));
        B.pfx_cap = n + 1;
    }
    launch_block_scan(h, B.pfxH, B.pfxS, 0, n);
    CU(cudaGetLastError());
    B.pfx_valid = true;
    return BS2E_OK;
}

// Band boundaries of the counted block: for the ascending n1 values xs[0..nx],
// rows[c * (nx + 1) + j] is the first row of channel c with n1 >= xs[j]
// (channel c holds rows [ch_start[c], ch_start[c + 1])), PH / PS the block's
// 1-based pointers there.
static bs2e_status band_bounds(bs2e_handle *h, const bs2e_config *cf,
                               const std::vector<int64_t> &xs, std::vector<int64_t> &rows,
                               std::vector<int64_t> &PH, std::vector<int64_t> &PS) {
    const BlockPlan &P = h->plan;
    const int n_ch = P.n_ch;
    const int64_t nx = (int64_t)xs.size() - 1;
    const int64_t m = (int64_t)n_ch * (nx + 1);
    rows.assign((size_t)m, 0);
    for (int c = 0; c < n_ch; ++c) {
        const int64_t lo = P.ch_start[c], hi = c + 1 < n_ch ? P.ch_start[c + 1] : P.n_config;
        int64_t r = lo;
        for (int64_t j = 0; j <= nx; ++j) {
            // n1 ascends within a channel (checked when the block was counted)
            int64_t a = r, b = hi;
            while (a < b) {
                const int64_t mid = a + (b - a) / 2;
                if (cf[mid].n1 < xs[(size_t)j]) a = mid + 1;
                else b = mid;
            }
            r = a;
            rows[(size_t)c * (nx + 1) + j] = r;
        }
    }
    PH.assign((size_t)m, 1);
    PS.assign((size_t)m, 1);
    if (m == 0) return BS2E_OK;
    TRY(ensure_prefix(h));
    if (2 * m > h->band_cap || !h->d_band_idx) {
        dfree(h->d_band_idx);
        dfree(h->d_band_val);
        h->band_cap = 0;
        const int64_t cap = std::max<int64_t>(2 * m, 2 * (kMaxCh + 1));
        CU(dalloc(&h->d_band_idx, (size_t)cap));
        CU(dalloc(&h->d_band_val, (size_t)cap));
        h->band_cap = cap;
    }
    CU(cudaMemcpyAsync(h->d_band_idx, rows.data(), sizeof(int64_t) * m, cudaMemcpyHostToDevice,
                       h->stream));
    launch_gather_i64(h, h->blk.pfxH, h->d_band_idx, m, h->d_band_val);
    launch_gather_i64(h, h->blk.pfxS, h->d_band_idx, m, h->d_band_val + m);
    CU(cudaMemcpyAsync(PH.data(), h->d_band_val, sizeof(int64_t) * m, cudaMemcpyDeviceToHost,
                       h->stream));
    CU(cudaMemcpyAsync(PS.data(), h->d_band_val + m, sizeof(int64_t) * m,
                       cudaMemcpyDeviceToHost, h->stream));
    return sync_check(h, "band bounds");
}

BS2E_API bs2e_status bs2e_block_band_count(bs2e_handle *h, const bs2e_config *configs,
                                           int64_t n_config, int64_t L, int64_t spin,
                                           int64_t full, int64_t n1_first, int64_t n1_count,
                                           int64_t *n_rows, int64_t *nnz_H, int64_t *nnz_S,
                                           int64_t *per_n1) {
    if (!h || n_config < 0 || !n_rows || !nnz_H || !nnz_S || n1_count < 0) return BS2E_ERR_ARG;
    Guard G(h);
    if (n1_count > (int64_t)1 << 24 || n1_first < -((int64_t)1 << 40) ||
        n1_first > ((int64_t)1 << 40))
        return fail(h, BS2E_ERR_ARG, "n1 range out of bounds");
    TRY(ensure_counted(h, configs, n_config, L, spin, full));
    std::vector<int64_t> rows, PH, PS, xs;
    const int64_t nx = per_n1 ? n1_count : 1;
    if (per_n1)
        for (int64_t j = 0; j <= n1_count; ++j) xs.push_back(n1_first + j);
    else
        xs = {n1_first, n1_first + n1_count};
    TRY(band_bounds(h, configs, xs, rows, PH, PS));
    const int n_ch = h->plan.n_ch;
    int64_t r = 0, eh = 0, es = 0;
    if (per_n1) memset(per_n1, 0, sizeof(int64_t) * 3 * (size_t)n1_count);
    for (int c = 0; c < n_ch; ++c) {
        const size_t o = (size_t)c * (nx + 1);
        r += rows[o + nx] - rows[o];
        eh += PH[o + nx] - PH[o];
        es += PS[o + nx] - PS[o];
        if (per_n1)
            for (int64_t j = 0; j < nx; ++j) {
                per_n1[3 * j] += rows[o + j + 1] - rows[o + j];
                per_n1[3 * j + 1] += PH[o + j + 1] - PH[o + j];
                per_n1[3 * j + 2] += PS[o + j + 1] - PS[o + j];
            }
    }
    *n_rows = r;
    *nnz_H = eh;
    *nnz_S = es;
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_block_fill_band(bs2e_handle *h, const bs2e_config *configs,
                                          int64_t n_config, int64_t L, int64_t spin,
                                          int64_t full, int64_t n1_first, int64_t n1_count,
                                          int64_t *rows_out, int64_t *H_index_ptr,
                                          int64_t *H_indices, double *H_data,
                                          int64_t *S_index_ptr, int64_t *S_indices,
                                          double *S_data, int64_t out_on_device) {
    if (!h || n_config < 0 || n1_count < 0) return BS2E_ERR_ARG;
    Guard G(h);
    if (n1_count > ((int64_t)1 << 40) || n1_first < -((int64_t)1 << 40) ||
        n1_first > ((int64_t)1 << 40))
        return fail(h, BS2E_ERR_ARG, "n1 range out of bounds");
    TRY(fill_ready(h, configs, n_config, L, spin, full));
    std::vector<int64_t> rows, PH, PS;
    TRY(band_bounds(h, configs, {n1_first, n1_first + n1_count}, rows, PH, PS));
    const int n_ch = h->plan.n_ch;
    std::vector<int> band(2 * (size_t)std::max(n_ch, 1), 0);
    std::vector<int64_t> boff(2 * ((size_t)n_ch + 1), 0);
    int64_t nr = 0;
    for (int c = 0; c < n_ch; ++c) {
        band[c] = (int)rows[2 * c];
        band[n_ch + c] = (int)nr;
        nr += rows[2 * c + 1] - rows[2 * c];
        boff[c + 1] = boff[c] + (PH[2 * c + 1] - PH[2 * c]);
        boff[n_ch + 2 + c] = boff[n_ch + 1 + c] + (PS[2 * c + 1] - PS[2 * c]);
    }
    const int64_t nH = boff[n_ch], nS = boff[2 * n_ch + 1];
    if (!H_index_ptr || !S_index_ptr || (nH > 0 && (!H_indices || !H_data)) ||
        (nS > 0 && (!S_indices || !S_data)))
        return fail(h, BS2E_ERR_ARG, "NULL output array");
    const bool dev = out_on_device != 0;
    if (dev) {
        if (!aligned(H_index_ptr, 8) || !aligned(S_index_ptr, 8) || !aligned(H_indices, 8) ||
            !aligned(S_indices, 8) || !aligned(H_data, 16) || !aligned(S_data, 16) ||
            !aligned(rows_out, 8))
            return fail(h, BS2E_ERR_ARG,
                        "device outputs: int64 arrays need 8-byte, data 16-byte alignment");
    }
    // host outputs: the band is cut into groups of whole channels (a band's
    // rows, and so its entries, are channel-major, so a group is one slice of
    // each output array); each group is filled into one of the two staging
    // areas while the copy stream moves the previous group to the host
    auto group_bytes = [&](int c0, int c1) {
        const int64_t hC = boff[c1] - boff[c0], sC = boff[n_ch + 1 + c1] - boff[n_ch + 1 + c0];
        return (8 * hC + 15) / 16 * 16 + 16 * hC + (8 * sC + 15) / 16 * 16 + 16 * sC;
    };
    std::vector<int> cut{0};
    if (!dev) {
        const int64_t total = group_bytes(0, n_ch);
        const int64_t target = std::min<int64_t>(
            h->stage_limit, std::max<int64_t>(total / 4, (int64_t)64 << 20));
        while (cut.back() < n_ch) {
            const int c0 = cut.back();
            int c1 = c0 + 1;
            if (group_bytes(c0, c1) > h->stage_limit)
                return fail(h, BS2E_ERR_ARG,
                            "band fill into host arrays: channel " + std::to_string(c0) +
                                " of the band needs " + std::to_string(group_bytes(c0, c1)) +
                                " bytes, more than a staging area; choose a narrower band or "
                                "raise bs2e_opts.stage_bytes");
            while (c1 < n_ch && group_bytes(c0, c1 + 1) <= target) ++c1;
            cut.push_back(c1);
        }
    }
    if (!h->d_band) CU(dalloc(&h->d_band, (size_t)2 * kMaxCh));
    if (!h->d_band_val) {
        CU(dalloc(&h->d_band_idx, (size_t)2 * (kMaxCh + 1)));
        CU(dalloc(&h->d_band_val, (size_t)2 * (kMaxCh + 1)));
        h->band_cap = 2 * (kMaxCh + 1);
    }
    // band pointers (and rows): the caller's arrays, or the handle's buffer
    int64_t *dHp = H_index_ptr, *dSp = S_index_ptr, *dRows = rows_out;
    if (!dev) {
        const int64_t need = 2 * (nr + 1) + (rows_out ? nr : 0);
        if (need > h->bptr_cap) {
            CU(cudaStreamSynchronize(h->stream));
            dfree(h->d_bptr);
            h->bptr_cap = 0;
            CU(dalloc(&h->d_bptr, (size_t)need));
            h->bptr_cap = need;
        }
        dHp = h->d_bptr;
        dSp = h->d_bptr + nr + 1;
        dRows = rows_out ? h->d_bptr + 2 * (nr + 1) : nullptr;
    }
    CU(cudaMemcpyAsync(h->d_band, band.data(), sizeof(int) * 2 * n_ch, cudaMemcpyHostToDevice,
                       h->stream));
    CU(cudaMemcpyAsync(h->d_band_val, boff.data(), sizeof(int64_t) * boff.size(),
                       cudaMemcpyHostToDevice, h->stream));
    launch_band_ptr(h, h->d_band, h->d_band_val, n_ch, nr, dHp, dSp, dRows);
    const int64_t a0 = std::max<int64_t>(n1_first, 1),
                  a1 = std::min<int64_t>(n1_first + n1_count - 1, h->g.N);
    FillRange r;
    r.row0 = 0;
    r.row1 = n_config;
    r.a0 = (int)a0;
    r.a1 = (int)a1;
    r.band = h->d_band;
    r.band_rows = nr;
    const bool any = nr > 0 && a1 >= a0;
    if (dev) {
        if (any) launch_block_fill(h, r, dHp, dSp, H_indices, (double2 *)H_data, S_indices,
                                   (double2 *)S_data);
        CU(cudaGetLastError());
        return sync_check(h, "block fill (band)");
    }
    const int n_group = (int)cut.size() - 1;
    int64_t most = 256;
    for (int g = 0; g < n_group; ++g) most = std::max(most, group_bytes(cut[g], cut[g + 1]));
    TRY(ensure_stage(h, most));
    TRY(ensure_copy_stream(h));
    struct Lay {
        size_t oHd, oSi, oSd;
        int64_t h0, hC, s0, sC;
    };
    auto lay = [&](int g) {
        Lay Ly;
        const int c0 = cut[g], c1 = cut[g + 1];
        Ly.h0 = boff[c0];
        Ly.hC = boff[c1] - boff[c0];
        Ly.s0 = boff[n_ch + 1 + c0];
        Ly.sC = boff[n_ch + 1 + c1] - Ly.s0;
        Ly.oHd = (size_t)((8 * Ly.hC + 15) / 16 * 16);
        Ly.oSi = Ly.oHd + 16 * (size_t)Ly.hC;
        Ly.oSd = Ly.oSi + (size_t)((8 * Ly.sC + 15) / 16 * 16);
        return Ly;
    };
    cudaError_t e = cudaSuccess;
    // fill of group g into area g % 2, after the copies out of that area
    // (group g - 2) are done
    auto fill = [&](int g) {
        const int b = g & 1;
        const Lay Ly = lay(g);
        unsigned char *base = h->d_stage[b];
        if (e == cudaSuccess && g >= 2) e = cudaStreamWaitEvent(h->stream, h->ev_copied[b], 0);
        FillRange rg = r;
        rg.Hbase = Ly.h0;
        rg.Sbase = Ly.s0;
        rg.ch0 = cut[g];
        rg.ch1 = cut[g + 1];
        if (e == cudaSuccess && any && (Ly.hC > 0 || Ly.sC > 0)) {
            launch_block_fill(h, rg, dHp, dSp, (int64_t *)base, (double2 *)(base + Ly.oHd),
                              (int64_t *)(base + Ly.oSi), (double2 *)(base + Ly.oSd));
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaEventRecord(h->ev_filled[b], h->stream);
    };
    auto cp = [&](cudaStream_t st, void *dst, const void *src, size_t bytes) {
        if (e == cudaSuccess && bytes)
            e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st);
    };
    // the fill of group g + 1 is queued before the copies of group g are
    // issued: a copy to pageable memory may block the host until it is done
    if (n_group > 0) fill(0);
    for (int g = 0; g < n_group && e == cudaSuccess; ++g) {
        if (g + 1 < n_group) fill(g + 1);
        const int b = g & 1;
        const Lay Ly = lay(g);
        const unsigned char *base = h->d_stage[b];
        if (e == cudaSuccess) e = cudaStreamWaitEvent(h->copy_stream, h->ev_filled[b], 0);
        cp(h->copy_stream, H_indices + Ly.h0, base, 8 * (size_t)Ly.hC);
        cp(h->copy_stream, H_data + 2 * Ly.h0, base + Ly.oHd, 16 * (size_t)Ly.hC);
        cp(h->copy_stream, S_indices + Ly.s0, base + Ly.oSi, 8 * (size_t)Ly.sC);
        cp(h->copy_stream, S_data + 2 * Ly.s0, base + Ly.oSd, 16 * (size_t)Ly.sC);
        if (e == cudaSuccess) e = cudaEventRecord(h->ev_copied[b], h->copy_stream);
    }
    cp(h->stream, H_index_ptr, dHp, 8 * (size_t)(nr + 1));
    cp(h->stream, S_index_ptr, dSp, 8 * (size_t)(nr + 1));
    if (rows_out) cp(h->stream, rows_out, dRows, 8 * (size_t)nr);
    cudaError_t e2 = cudaStreamSynchronize(h->copy_stream);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) {
        cudaStreamSynchronize(h->stream);
        return fail(h, e == cudaErrorMemoryAllocation ? BS2E_ERR_NOMEM : BS2E_ERR_CUDA,
                    std::string("block fill (band, streamed): ") + cudaGetErrorString(e));
    }
    return sync_check(h, "block fill (band)");
}

BS2E_API bs2e_status bs2e_set_block_cache(bs2e_handle *h, int64_t n_blocks) {
    if (!h) return BS2E_ERR_ARG;
    Guard G(h);
    if (n_blocks < 0 || n_blocks > kBlockCache)
        return fail(h, BS2E_ERR_ARG, "block cache size must be 0..16");
    h->cache_max = (int)n_blocks;
    if (h->parked.size() > (size_t)n_blocks) {
        CU(cudaStreamSynchronize(h->stream));
        while (h->parked.size() > (size_t)n_blocks) {
            free_block(h->parked.back().first);
            h->parked.pop_back();
        }
    }
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_block_fill(bs2e_handle *h, const bs2e_config *configs,
                                     int64_t n_config, int64_t L, int64_t full, const double *H1p,
                                     int64_t n_l, const double *S, int64_t *H_index_ptr,
                                     int64_t *H_indices, double *H_data, int64_t *S_index_ptr,
                                     int64_t *S_indices, double *S_data) {
    if (!h) return BS2E_ERR_ARG;
    if (H1p || S) {
        if (!H1p || !S) return BS2E_ERR_ARG;
        bs2e_status st = bs2e_set_one_body(h, H1p, n_l, S);
        if (st != BS2E_OK) return st;
    }
    return bs2e_block_fill_ex(h, configs, n_config, L, 0, full, H_index_ptr, H_indices, H_data,
                              S_index_ptr, S_indices, S_data, 0);
}

BS2E_API bs2e_status bs2e_radial_dipole(bs2e_handle *h, int64_t gauge, double *r_mat,
                                        double *dr_mat, double *r_inv_mat) {
    if (!h || (gauge != 0 && gauge != 1)) return BS2E_ERR_ARG;
    Guard G(h);
    if (!h->slater_done) return fail(h, BS2E_ERR_STATE, "bs2e_slater has not run (tabulation)");
    const Radial &g = h->g;
    const int N = g.N, W = g.W, k = g.k;
    dfree(h->d_dM1);
    dfree(h->d_dM2);
    CU(dalloc(&h->d_dM1, (size_t)N * W));
    if (gauge == 1) CU(dalloc(&h->d_dM2, (size_t)N * W));
    launch_radial_dip(h, (int)gauge);
    TRY(sync_check(h, "radial dipole"));
    h->dip_gauge = (int)gauge;
    h->dip_kind = gauge == 0 ? 1 : 2;  // <r> is real, -i<d/dr> and -i<1/r> imaginary
    double *outs[2] = {gauge == 0 ? r_mat : dr_mat, gauge == 1 ? r_inv_mat : nullptr};
    double2 *src[2] = {h->d_dM1, h->d_dM2};
    for (int m = 0; m < 2; ++m) {
        if (!outs[m] || !src[m]) continue;
        std::vector<double2> b((size_t)N * W);
        CU(cudaMemcpy(b.data(), src[m], b.size() * sizeof(double2), cudaMemcpyDeviceToHost));
        memset(outs[m], 0, sizeof(double) * 2 * (size_t)N * N);
        for (int x = 0; x < N; ++x)
            for (int d = 0; d < W; ++d) {
                int y = x + d - (k - 1);
                if (y < 0 || y >= N) continue;
                size_t o = ((size_t)y * N + x) * 2;
                outs[m][o] = b[(size_t)x * W + d].x;
                outs[m][o + 1] = b[(size_t)x * W + d].y;
            }
    }
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_set_radial_dipole(bs2e_handle *h, int64_t gauge, const double *r_mat,
                                            const double *dr_mat, const double *r_inv_mat) {
    if (!h || (gauge != 0 && gauge != 1)) return BS2E_ERR_ARG;
    if ((gauge == 0 && !r_mat) || (gauge == 1 && (!dr_mat || !r_inv_mat))) return BS2E_ERR_ARG;
    Guard G(h);
    const Radial &g = h->g;
    const int N = g.N, W = g.W, k = g.k;
    const double *ins[2] = {gauge == 0 ? r_mat : dr_mat, gauge == 1 ? r_inv_mat : nullptr};
    dfree(h->d_dM1);
    dfree(h->d_dM2);
    double2 **dst[2] = {&h->d_dM1, &h->d_dM2};
    bool all_re = true, all_im = true;  // every band value real / imaginary
    for (int m = 0; m < 2; ++m) {
        if (!ins[m]) continue;
        std::vector<double2> b((size_t)N * W, make_double2(0.0, 0.0));
        for (int x = 0; x < N; ++x)
            for (int d = 0; d < W; ++d) {
                int y = x + d - (k - 1);
                if (y < 0 || y >= N) continue;
                size_t o = ((size_t)y * N + x) * 2;
                b[(size_t)x * W + d] = make_double2(ins[m][o], ins[m][o + 1]);
                all_re = all_re && ins[m][o + 1] == 0.0;
                all_im = all_im && ins[m][o] == 0.0;
            }
        CU(dalloc(dst[m], b.size()));
        CU(cudaMemcpy(*dst[m], b.data(), b.size() * sizeof(double2), cudaMemcpyHostToDevice));
    }
    h->dip_gauge = (int)gauge;
    h->dip_kind = all_re ? 1 : (all_im ? 2 : 0);
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_dip_block_count(bs2e_handle *h, const bs2e_config *rows, int64_t n_rows,
                                          int64_t L1, int64_t M1, int64_t pi1,
                                          const bs2e_config *cols, int64_t n_cols, int64_t L2,
                                          int64_t M2, int64_t pi2, int64_t q, int64_t compute,
                                          int64_t *nnz) {
    if (!h || !nnz) return BS2E_ERR_ARG;
    Guard G(h);
    DipDev D;
    bool empty;
    return dip_prepare(h, rows, n_rows, L1, M1, pi1, cols, n_cols, L2, M2, pi2, q, compute, D,
                       empty, *nnz);
}

BS2E_API bs2e_status bs2e_dip_block_fill(bs2e_handle *h, const bs2e_config *rows, int64_t n_rows,
                                         int64_t L1, int64_t M1, int64_t pi1,
                                         const bs2e_config *cols, int64_t n_cols, int64_t L2,
                                         int64_t M2, int64_t pi2, int64_t q, int64_t compute,
                                         int64_t *index_ptr, int64_t *indices, double *data,
                                         int64_t out_on_device) {
    if (!h || !index_ptr) return BS2E_ERR_ARG;
    Guard G(h);
    DipDev D;
    bool empty;
    int64_t nnz = 0;
    TRY(dip_prepare(h, rows, n_rows, L1, M1, pi1, cols, n_cols, L2, M2, pi2, q, compute, D, empty,
                    nnz));
    const bool dev = out_on_device != 0;
    if (dev && (!aligned(index_ptr, 8) || !aligned(indices, 8) || !aligned(data, 16)))
        return fail(h, BS2E_ERR_ARG, "device outputs: int64 arrays need 8-byte, data 16-byte alignment");
    if (empty) {
        std::vector<int64_t> ones((size_t)n_rows + 1, 1);
        if (dev)
            CU(cudaMemcpy(index_ptr, ones.data(), sizeof(int64_t) * ones.size(),
                          cudaMemcpyHostToDevice));
        else
            memcpy(index_ptr, ones.data(), sizeof(int64_t) * ones.size());
        return BS2E_OK;
    }
    if (nnz > 0 && (!indices || !data)) return fail(h, BS2E_ERR_ARG, "NULL output array");
    int64_t *dp = index_ptr, *di = indices;
    double2 *dd = (double2 *)data;
    if (!dev) {
        CU(dalloc(&dp, (size_t)n_rows + 1));
        CU(dalloc(&di, (size_t)nnz));
        CU(dalloc(&dd, (size_t)nnz));
    }
    CU(grow(&h->d_dip_part, h->dip_part_cap, (n_rows + 4095) / 4096 + 4));
    scan_one(h, h->d_dip_cnt, n_rows, h->d_dip_part, dp);
    launch_dip_fill(h, D, dp, di, dd);
    bs2e_status st = BS2E_OK;
    if (!dev) {
        cudaError_t e = cudaMemcpyAsync(index_ptr, dp, sizeof(int64_t) * (n_rows + 1),
                                        cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess && nnz)
            e = cudaMemcpyAsync(indices, di, sizeof(int64_t) * nnz, cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess && nnz)
            e = cudaMemcpyAsync(data, dd, sizeof(double2) * nnz, cudaMemcpyDeviceToHost, h->stream);
        if (e != cudaSuccess) st = fail(h, BS2E_ERR_CUDA, cudaGetErrorString(e));
    }
    bs2e_status st2 = sync_check(h, "dipole fill");
    if (!dev) {
        cudaFree(dp);
        cudaFree(di);
        cudaFree(dd);
    }
    return st != BS2E_OK ? st : st2;
}

BS2E_API bs2e_status bs2e_stream(bs2e_handle *h, void **stream) {
    if (!h || !stream) return BS2E_ERR_ARG;
    *stream = (void *)h->stream;
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_set_stream_priority(bs2e_handle *h, int64_t priority) {
    if (!h) return BS2E_ERR_ARG;
    Guard g(h);
    int lo = 0, hi = 0;  // CUDA's range: lo is the lowest priority, hi the highest
    CU(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    if (priority > lo || priority < hi)
        return fail(h, BS2E_ERR_ARG, "set_stream_priority: outside the device's priority range");
    cudaStream_t s = nullptr;
    CU(cudaStreamSynchronize(h->stream));
    CU(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, (int)priority));
    cudaStreamDestroy(h->stream);
    h->stream = s;
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_launch_count(const bs2e_handle *h, int64_t *count) {
    if (!h || !count) return BS2E_ERR_ARG;
    *count = h->launches;
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_synchronize(bs2e_handle *h) {
    if (!h) return BS2E_ERR_ARG;
    Guard G(h);
    return sync_check(h, "synchronize");
}

}  // extern "C"

// CSR_mv / CSR_T_mv / CSR_mv_sym (sparse_array_tools.f90:966-1074).
BS2E_API bs2e_status bs2e_csr_mv(bs2e_handle *h, int64_t op, int64_t n_rows, int64_t n_cols,
                                 int64_t nnz, const int64_t *index_ptr, const int64_t *indices,
                                 const double *data, const double *x, double *y,
                                 int64_t on_device) {
    if (!h) return BS2E_ERR_ARG;
    Guard g(h);
    if (op < 0 || op > 2) return fail(h, BS2E_ERR_ARG, "csr_mv: op must be 0 (N), 1 (T) or 2 (sym)");
    if (n_rows < 0 || n_cols < 0 || nnz < 0 || n_rows > ((int64_t)1 << 34))
        return fail(h, BS2E_ERR_ARG, "csr_mv: negative or too large sizes");
    if (op == 2 && n_rows != n_cols)
        return fail(h, BS2E_ERR_ARG, "csr_mv: the symmetric product needs a square matrix");
    const int64_t n_out = op == 1 ? n_cols : n_rows, n_in = op == 1 ? n_rows : n_cols;
    if (!index_ptr || !x || !y || (nnz > 0 && (!indices || !data)))
        return fail(h, BS2E_ERR_ARG, "csr_mv: NULL array");
    if (!h->d_mv_bad) CU(dalloc(&h->d_mv_bad, 1));
    CU(cudaMemsetAsync(h->d_mv_bad, 0, sizeof(int), h->stream));
    const int64_t *dp = index_ptr, *di = indices;
    const double2 *dA = (const double2 *)data, *dx = (const double2 *)x;
    double2 *dy = (double2 *)y;
    if (on_device && (!aligned(index_ptr, 8) || !aligned(indices, 8) || !aligned(data, 16) ||
                      !aligned(x, 16) || !aligned(y, 16)))
        return fail(h, BS2E_ERR_ARG, "csr_mv: int64 arrays need 8-byte, complex arrays 16-byte alignment");
    if (!on_device) {
        if (index_ptr[n_rows] - 1 != nnz)
            return fail(h, BS2E_ERR_ARG, "csr_mv: index_ptr(n_rows+1) - 1 differs from nnz");
        CU(grow(&h->d_mv_ptr, h->mv_ptr_cap, n_rows + 1));
        CU(grow(&h->d_mv_idx, h->mv_idx_cap, nnz));
        CU(grow(&h->d_mv_A, h->mv_A_cap, nnz));
        CU(grow(&h->d_mv_x, h->mv_x_cap, n_in));
        CU(grow(&h->d_mv_y, h->mv_y_cap, n_out));
        CU(cudaMemcpyAsync(h->d_mv_ptr, index_ptr, 8 * (size_t)(n_rows + 1),
                           cudaMemcpyHostToDevice, h->stream));
        if (nnz > 0) {
            CU(cudaMemcpyAsync(h->d_mv_idx, indices, 8 * (size_t)nnz, cudaMemcpyHostToDevice,
                               h->stream));
            CU(cudaMemcpyAsync(h->d_mv_A, data, 16 * (size_t)nnz, cudaMemcpyHostToDevice,
                               h->stream));
        }
        if (n_in > 0)
            CU(cudaMemcpyAsync(h->d_mv_x, x, 16 * (size_t)n_in, cudaMemcpyHostToDevice,
                               h->stream));
        dp = h->d_mv_ptr;
        di = h->d_mv_idx;
        dA = h->d_mv_A;
        dx = h->d_mv_x;
        dy = h->d_mv_y;
    }
    launch_csr_mv(h, (int)op, n_rows, n_cols, nnz, dp, di, dA, dx, dy, h->d_mv_bad);
    CU(cudaGetLastError());
    if (!on_device && n_out > 0)
        CU(cudaMemcpyAsync(y, dy, 16 * (size_t)n_out, cudaMemcpyDeviceToHost, h->stream));
    int bad = 0;
    CU(cudaMemcpyAsync(&bad, h->d_mv_bad, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    TRY(sync_check(h, "csr_mv"));
    if (bad & 1) return fail(h, BS2E_ERR_ARG, "csr_mv: index_ptr out of range or decreasing");
    if (bad & 2) return fail(h, BS2E_ERR_ARG, "csr_mv: column index outside 1..n_cols");
    return BS2E_OK;
}

// CS_from_block / CSR_from_block (block_tools.f90:153-234).
BS2E_API bs2e_status bs2e_csr_from_blocks(bs2e_handle *h, int64_t n_rb, int64_t n_cb,
                                          const int64_t *shapes, const int64_t *nnz,
                                          const int64_t *const *index_ptr,
                                          const int64_t *const *indices,
                                          const double *const *data, int64_t *out_index_ptr,
                                          int64_t *out_indices, double *out_data,
                                          int64_t on_device) {
    if (!h) return BS2E_ERR_ARG;
    Guard g(h);
    if (n_rb < 1 || n_cb < 1 || n_rb * n_cb > (1 << 20) || !shapes || !nnz || !out_index_ptr)
        return fail(h, BS2E_ERR_ARG, "csr_from_blocks: bad block grid or NULL array");
    const int64_t nb = n_rb * n_cb;
    std::vector<int64_t> row0(n_rb + 1, 0);
    int64_t tot = 0;
    for (int64_t i = 0; i < n_rb; ++i) {
        const int64_t rows = shapes[2 * i];  // block (i, 1) gives the row count
        if (rows < 0) return fail(h, BS2E_ERR_ARG, "csr_from_blocks: negative shape");
        for (int64_t j = 0; j < n_cb; ++j) {
            const int64_t b = i + n_rb * j;
            if (shapes[2 * b] < 0 || shapes[2 * b + 1] < 0 || nnz[b] < 0)
                return fail(h, BS2E_ERR_ARG, "csr_from_blocks: negative shape or nnz");
            if (nnz[b] > 0 && shapes[2 * b] != rows)
                return fail(h, BS2E_ERR_ARG, "csr_from_blocks: blocks of one block row differ in rows");
            if (nnz[b] > 0 && (!index_ptr || !indices || !data || !index_ptr[b] || !indices[b] || !data[b]))
                return fail(h, BS2E_ERR_ARG, "csr_from_blocks: NULL array of a non-empty block");
            tot += nnz[b];
        }
        row0[i + 1] = row0[i] + rows;
    }
    const int64_t n_rows = row0[n_rb];
    if (tot > 0 && (!out_indices || !out_data)) return fail(h, BS2E_ERR_ARG, "csr_from_blocks: NULL output");
    if (on_device && (!aligned(out_index_ptr, 8) || !aligned(out_indices, 8) || !aligned(out_data, 16)))
        return fail(h, BS2E_ERR_ARG, "csr_from_blocks: int64 arrays need 8-byte, data 16-byte alignment");
    if (n_rows == 0) {
        if (tot > 0) return fail(h, BS2E_ERR_ARG, "csr_from_blocks: entries in blocks without rows");
        const int64_t one = 1;
        if (!on_device) {
            out_index_ptr[0] = 1;
            return BS2E_OK;
        }
        CU(cudaMemcpy(out_index_ptr, &one, 8, cudaMemcpyHostToDevice));
        return BS2E_OK;
    }
    std::vector<CatBlock> cb(nb);
    // host operands are staged: one device area for every non-empty block
    std::vector<void *> staged;
    auto cleanup = [&]() {
        for (void *p : staged) cudaFree(p);
    };
    for (int64_t i = 0; i < n_rb; ++i) {
        int64_t col = 0;
        for (int64_t j = 0; j < n_cb; ++j) {
            const int64_t b = i + n_rb * j;
            CatBlock &B = cb[b];
            B.nnz = nnz[b];
            B.n_cols = shapes[2 * b + 1];
            B.col0 = col;
            B.ptr = nullptr;
            B.idx = nullptr;
            B.data = nullptr;
            col += shapes[2 * b + 1];
            if (nnz[b] <= 0) continue;
            if (on_device) {
                if (!aligned(index_ptr[b], 8) || !aligned(indices[b], 8) || !aligned(data[b], 16)) {
                    cleanup();
                    return fail(h, BS2E_ERR_ARG, "csr_from_blocks: int64 arrays need 8-byte, data 16-byte alignment");
                }
                B.ptr = index_ptr[b];
                B.idx = indices[b];
                B.data = (const double2 *)data[b];
                continue;
            }
            const int64_t rows = shapes[2 * b];
            char *d = nullptr;
            // complex data 16-byte aligned after the int64 pointers and columns
            const size_t o_dat = (8 * (size_t)(rows + 1 + nnz[b]) + 15) / 16 * 16;
            const size_t bytes = o_dat + 16 * (size_t)nnz[b];
            cudaError_t e = cudaMalloc(&d, bytes);
            if (e != cudaSuccess) {
                cleanup();
                return fail(h, BS2E_ERR_NOMEM, "csr_from_blocks: staging");
            }
            staged.push_back(d);
            int64_t *dp = (int64_t *)d, *di = dp + rows + 1;
            double2 *dd = (double2 *)(d + o_dat);
            e = cudaMemcpyAsync(dp, index_ptr[b], 8 * (size_t)(rows + 1), cudaMemcpyHostToDevice, h->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(di, indices[b], 8 * (size_t)nnz[b], cudaMemcpyHostToDevice, h->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(dd, data[b], 16 * (size_t)nnz[b], cudaMemcpyHostToDevice, h->stream);
            if (e != cudaSuccess) {
                cudaStreamSynchronize(h->stream);
                cleanup();
                return fail(h, BS2E_ERR_CUDA, cudaGetErrorString(e));
            }
            B.ptr = dp;
            B.idx = di;
            B.data = dd;
        }
    }
    // device tables, counts, scan partials, flag, and (host mode) outputs
    const size_t nparts = (size_t)(n_rows + 4095) / 4096 + 4;
    size_t tbytes = sizeof(CatBlock) * nb + 8 * (size_t)(n_rb + 1) + 8 * (size_t)(n_rows + 1) +
                    8 * nparts + 16;
    size_t obytes = on_device ? 0 : 8 * (size_t)(n_rows + 1) + 24 * (size_t)tot + 16;
    char *t = nullptr;
    cudaError_t e = cudaMalloc(&t, tbytes + obytes);
    if (e != cudaSuccess) {
        cleanup();
        return fail(h, BS2E_ERR_NOMEM, "csr_from_blocks: work area");
    }
    staged.push_back(t);
    CatBlock *d_cb = (CatBlock *)t;
    int64_t *d_row0 = (int64_t *)(t + sizeof(CatBlock) * nb);
    int64_t *d_cnt = d_row0 + n_rb + 1;
    int64_t *d_part = d_cnt + n_rows + 1;
    int *d_bad = (int *)(d_part + nparts);
    int64_t *optr = out_index_ptr, *oidx = out_indices;
    double2 *odat = (double2 *)out_data;
    if (!on_device) {
        char *o = t + tbytes;
        optr = (int64_t *)o;
        oidx = optr + n_rows + 1;
        odat = (double2 *)(((uintptr_t)(oidx + tot) + 15) & ~(uintptr_t)15);
    }
    e = cudaMemcpyAsync(d_cb, cb.data(), sizeof(CatBlock) * nb, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_row0, row0.data(), 8 * (size_t)(n_rb + 1), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_bad, 0, sizeof(int), h->stream);
    CatArgs A;
    A.blocks = d_cb;
    A.row0 = d_row0;
    A.n_rb = (int)n_rb;
    A.n_cb = (int)n_cb;
    A.n_rows = n_rows;
    if (e == cudaSuccess) {
        launch_cat(h, A, d_cnt, d_part, optr, nullptr, nullptr, d_bad, false);
        e = cudaGetLastError();
    }
    int64_t last = 1;
    int bad = 0;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&last, optr + n_rows, 8, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
        cleanup();
        return fail(h, BS2E_ERR_CUDA, cudaGetErrorString(e));
    }
    if (bad || last - 1 != tot) {
        cleanup();
        return fail(h, BS2E_ERR_ARG, "csr_from_blocks: a block index_ptr is out of range or "
                                     "disagrees with its nnz");
    }
    if (tot > 0) {
        launch_cat(h, A, nullptr, nullptr, optr, oidx, odat, d_bad, true);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && !on_device) {
        e = cudaMemcpyAsync(out_index_ptr, optr, 8 * (size_t)(n_rows + 1), cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess && tot > 0)
            e = cudaMemcpyAsync(out_indices, oidx, 8 * (size_t)tot, cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess && tot > 0)
            e = cudaMemcpyAsync(out_data, odat, 16 * (size_t)tot, cudaMemcpyDeviceToHost, h->stream);
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cleanup();
    if (e != cudaSuccess) return fail(h, BS2E_ERR_CUDA, cudaGetErrorString(e));
    if (bad & 2) return fail(h, BS2E_ERR_ARG, "csr_from_blocks: a column index exceeds its block's width");
    return BS2E_OK;
}
