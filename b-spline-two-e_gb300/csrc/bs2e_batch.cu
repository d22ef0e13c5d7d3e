// bs2e_batch.cu -- the radial stage of many bases at once.
//
// A ragged batch (each basis with its own order, spline count, knot grid and
// multipole range) runs bs2e_slater + bs2e_rk of every handle as four
// persistent kernels (tabulation, moments, pair totals, R^k store of the
// FP64 and of the mixed problems), each draining one work queue that spans
// all problems, so small problems do not leave the GPU idle and there is one
// launch per stage instead of one per problem and stage.  The first run tunes
// the R^k stage (threads per CTA, items taken per queue access) by timing
// each candidate; the stages are then captured once in a CUDA graph and later
// runs replay it.  Results are
// bit-identical to the per-handle path: both run the same device functions.
//
// Reference: setup_Slater_integrals and compute_R_k_map
// (src/mat_els/mat_els.f90:172-292, src/tools/sparse_array_tools.f90:452-493),
// which the reference runs for one basis per basis_setup invocation.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "bs2e_internal.h"

using namespace bs2e;

struct bs2e_batch {
    std::vector<bs2e_handle *> hs;  // in queue order (largest R^k store first)
    int device = 0;
    cudaStream_t stream = nullptr;
    RadialDev *d_probs = nullptr;
    int64_t *d_off = nullptr;                // kStages x (n + 1)
    unsigned long long *d_counter = nullptr;  // kStages counters
    std::vector<int64_t> off[5];
    size_t smem[5] = {0, 0, 0, 0, 0};
    int threads[5] = {128, 256, 256, 256, 256};
    int grid[5] = {1, 1, 1, 1, 1};
    int chunk = 1;
    int persistent = 1;  // R^k stage: queue-draining CTAs (1) or one CTA per chunk (0)
    int sms = 0;
    bool tuned = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t launches = 0;
    std::string err;
};

namespace {

constexpr int kTotThreads = 256;
constexpr int kStages = 5;  // tabulate, moments, totals, R^k FP64, R^k mixed

// Locks every handle of the batch (in address order, so two batches sharing
// handles cannot deadlock).
struct LockAll {
    std::vector<std::unique_lock<std::mutex>> lk;
    explicit LockAll(const std::vector<bs2e_handle *> &hs) {
        std::vector<bs2e_handle *> s(hs);
        std::sort(s.begin(), s.end());
        for (bs2e_handle *h : s) lk.emplace_back(h->mu);
    }
};

bs2e_status bfail(bs2e_batch *b, bs2e_status st, const std::string &m) {
    b->err = m;
    for (bs2e_handle *h : b->hs) h->err = m;  // readable through any handle
    return st;
}

#define BCU(call)                                                                             \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return bfail(b, e_ == cudaErrorMemoryAllocation ? BS2E_ERR_NOMEM : BS2E_ERR_CUDA, \
                         std::string(#call) + ": " + cudaGetErrorString(e_));                 \
    } while (0)

// Persistent grid of a stage: every CTA the SMs hold at once (no more than
// there are items).  Also sets the kernel's shared-memory limit, so it is
// called outside graph capture.
void set_grid(bs2e_batch *b, int stage, int chunk = 1, int persistent = 1) {
    int per = radial_batch_blocks_per_sm(stage, b->threads[stage], b->smem[stage]);
    if (per < 1) per = 1;
    int64_t items = b->off[stage].back();
    if (!persistent) {
        b->grid[stage] = (int)std::max<int64_t>((items + chunk - 1) / chunk, 1);
        return;
    }
    b->grid[stage] = (int)std::min<int64_t>((int64_t)per * b->sms, std::max<int64_t>(items, 1));
}

void enqueue_stage(bs2e_batch *b, int stage, int chunk, int persistent = 1) {
    const int n = (int)b->hs.size();
    launch_radial_batch(b->stream, stage, b->grid[stage], b->threads[stage], b->smem[stage],
                        b->d_probs, b->d_off + (size_t)stage * (n + 1), n, b->d_counter + stage,
                        stage >= 3 ? chunk : 1, stage >= 3 ? persistent : 1);
    b->launches++;
}

void enqueue_all(bs2e_batch *b) {
    cudaMemsetAsync(b->d_counter, 0, kStages * sizeof(unsigned long long), b->stream);
    for (int st = 0; st < kStages; ++st)
        if (b->off[st].back() > 0) enqueue_stage(b, st, b->chunk, b->persistent);
}

// Times the R^k stage for each candidate (threads per CTA x work
// distribution: a queue drained by resident CTAs taking 1, 2 or 8 tiles per
// access, or one CTA per 1 or 4 tiles) and keeps the fastest.
bs2e_status tune(bs2e_batch *b) {
    struct Cand {
        int persistent, chunk;
    };
    const int cand_threads[2] = {128, 256};
    const int ts = b->off[3].back() > 0 ? 3 : 4;  // the R^k stage that is timed
    const Cand cand[5] = {{1, 1}, {1, 2}, {1, 8}, {0, 1}, {0, 4}};
    cudaEvent_t e0, e1;
    BCU(cudaEventCreate(&e0));
    BCU(cudaEventCreate(&e1));
    float best = 1e30f;
    int bt = 256, bc = 1, bp = 1;
    for (int t : cand_threads)
        for (const Cand &c : cand) {
            b->threads[ts] = t;
            set_grid(b, ts, c.chunk, c.persistent);
            BCU(cudaMemsetAsync(b->d_counter + ts, 0, sizeof(unsigned long long), b->stream));
            BCU(cudaEventRecord(e0, b->stream));
            enqueue_stage(b, ts, c.chunk, c.persistent);
            BCU(cudaEventRecord(e1, b->stream));
            BCU(cudaEventSynchronize(e1));
            BCU(cudaGetLastError());
            float ms = 0.f;
            BCU(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best) {
                best = ms;
                bt = t;
                bc = c.chunk;
                bp = c.persistent;
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->threads[3] = b->threads[4] = bt;
    b->chunk = bc;
    b->persistent = bp;
    set_grid(b, 3, bc, bp);
    set_grid(b, 4, bc, bp);
    b->tuned = true;
    // the other R^k stage, if the batch has one, runs once with the choice
    if (ts == 3 && b->off[4].back() > 0) {
        BCU(cudaMemsetAsync(b->d_counter + 4, 0, sizeof(unsigned long long), b->stream));
        enqueue_stage(b, 4, bc, bp);
        BCU(cudaGetLastError());
    }
    return BS2E_OK;
}

void mark_done(bs2e_batch *b) {
    for (bs2e_handle *h : b->hs) {
        h->slater_done = true;
        std::fill(h->rk_done.begin(), h->rk_done.end(), 1);
    }
}

}  // namespace

BS2E_API bs2e_status bs2e_batch_create(bs2e_handle *const *handles, int64_t n, bs2e_batch **out) {
    if (!out || !handles || n < 1 || n > (1 << 20)) return BS2E_ERR_ARG;
    *out = nullptr;
    std::vector<bs2e_handle *> hs(handles, handles + n);
    for (bs2e_handle *h : hs)
        if (!h) return BS2E_ERR_ARG;
    {
        std::vector<bs2e_handle *> s(hs);
        std::sort(s.begin(), s.end());
        if (std::adjacent_find(s.begin(), s.end()) != s.end()) return BS2E_ERR_ARG;
    }
    const int dev = hs[0]->device;
    for (bs2e_handle *h : hs)
        if (h->device != dev) {
            hs[0]->err = "batch: every handle must be on the same device";
            return BS2E_ERR_ARG;
        }
    bs2e_batch *b = new (std::nothrow) bs2e_batch();
    if (!b) return BS2E_ERR_NOMEM;
    // largest R^k store first: the long items start early
    std::stable_sort(hs.begin(), hs.end(), [](const bs2e_handle *x, const bs2e_handle *y) {
        return (int64_t)x->g.N * x->g.N * x->g.tile > (int64_t)y->g.N * y->g.N * y->g.tile;
    });
    b->hs = hs;
    b->device = dev;
    bs2e_status st = BS2E_OK;
    {
        LockAll L(b->hs);
        cudaSetDevice(dev);
        auto run = [&]() -> bs2e_status {
            cudaDeviceProp prop;
            BCU(cudaGetDeviceProperties(&prop, dev));
            b->sms = prop.multiProcessorCount;
            BCU(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
            std::vector<RadialDev> probs;
            for (int s = 0; s < kStages; ++s) b->off[s].assign(1, 0);
            for (bs2e_handle *h : b->hs) {
                BCU(cudaStreamSynchronize(h->stream));
                const Radial &g = h->g;
                const bool mixed = h->precision == BS2E_PREC_MIXED;
                if (mixed) {
                    if (!h->d_Rf) BCU(cudaMalloc(&h->d_Rf, sizeof(float2) * (size_t)g.N * g.N * g.tile));
                    if (!h->d_Rexp) BCU(cudaMalloc(&h->d_Rexp, sizeof(int) * (size_t)g.N * g.N * g.K1));
                } else if (!h->d_R) {
                    BCU(cudaMalloc(&h->d_R, sizeof(double) * (size_t)g.N * g.N * g.tile));
                }
                const int rs = mixed ? 4 : 3;
                b->smem[rs] = std::max(b->smem[rs], rk_store_smem(g, mixed));
                b->smem[1] = std::max(b->smem[1], moments_smem(g));
                probs.push_back(radial_dev(h));
                const int64_t tiles = (int64_t)g.N * g.N;
                const int64_t items[kStages] = {
                    g.n_iv, (int64_t)g.n_iv * g.K1,
                    ((int64_t)2 * g.K1 * g.N * g.W + kTotThreads - 1) / kTotThreads,
                    mixed ? 0 : tiles, mixed ? tiles : 0};
                for (int s = 0; s < kStages; ++s) b->off[s].push_back(b->off[s].back() + items[s]);
            }
            b->threads[2] = kTotThreads;
            const size_t nn = b->hs.size();
            BCU(cudaMalloc(&b->d_probs, sizeof(RadialDev) * nn));
            BCU(cudaMalloc(&b->d_off, sizeof(int64_t) * kStages * (nn + 1)));
            BCU(cudaMalloc(&b->d_counter, kStages * sizeof(unsigned long long)));
            BCU(cudaMemcpy(b->d_probs, probs.data(), sizeof(RadialDev) * nn, cudaMemcpyHostToDevice));
            for (int s = 0; s < kStages; ++s)
                BCU(cudaMemcpy(b->d_off + (size_t)s * (nn + 1), b->off[s].data(),
                               sizeof(int64_t) * (nn + 1), cudaMemcpyHostToDevice));
            for (int s = 0; s < kStages; ++s) set_grid(b, s);
            BCU(cudaGetLastError());
            return BS2E_OK;
        };
        st = run();
    }
    if (st != BS2E_OK) {
        bs2e_batch_destroy(b);
        return st;
    }
    *out = b;
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_batch_run(bs2e_batch *b) {
    if (!b) return BS2E_ERR_ARG;
    LockAll L(b->hs);
    cudaSetDevice(b->device);
    for (bs2e_handle *h : b->hs) BCU(cudaStreamSynchronize(h->stream));
    if (!b->tuned) {
        // first run: stages 0-2 eagerly, then every candidate of an R^k stage
        // (each a complete pass), the other R^k stage once, then the graph
        BCU(cudaMemsetAsync(b->d_counter, 0, kStages * sizeof(unsigned long long), b->stream));
        for (int s = 0; s < 3; ++s) enqueue_stage(b, s, 1);
        BCU(cudaGetLastError());
        bs2e_status st = tune(b);
        if (st != BS2E_OK) return st;
        BCU(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        enqueue_all(b);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (e != cudaSuccess) return bfail(b, BS2E_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        b->graph = g;
        BCU(cudaGraphInstantiate(&b->exec, b->graph, 0));
        BCU(cudaStreamSynchronize(b->stream));
        mark_done(b);
        return BS2E_OK;
    }
    BCU(cudaGraphLaunch(b->exec, b->stream));
    for (int st = 0; st < kStages; ++st) b->launches += b->off[st].back() > 0 ? 1 : 0;
    BCU(cudaStreamSynchronize(b->stream));
    BCU(cudaGetLastError());
    mark_done(b);
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_batch_tuning(const bs2e_batch *b, int64_t *rk_threads, int64_t *chunk,
                                       int64_t *graph_ready, int64_t *launches) {
    if (!b) return BS2E_ERR_ARG;
    if (rk_threads) *rk_threads = b->threads[3];
    if (chunk) *chunk = b->persistent ? b->chunk : -b->chunk;
    if (graph_ready) *graph_ready = b->exec ? 1 : 0;
    if (launches) *launches = b->launches;
    return BS2E_OK;
}

BS2E_API bs2e_status bs2e_batch_destroy(bs2e_batch *b) {
    if (!b) return BS2E_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->d_probs) cudaFree(b->d_probs);
    if (b->d_off) cudaFree(b->d_off);
    if (b->d_counter) cudaFree(b->d_counter);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return BS2E_OK;
}
