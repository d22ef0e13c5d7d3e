// bs2e_noalloc.cu -- R^k lookups that allocate no device memory.
//
// bs2e_rk_get_batch stages the caller's keys and the looked-up values through
// device buffers it allocates (and frees) on every call.  Some callers can't
// afford that: a caller that has filled HBM with CSR blocks can't risk an
// allocation failing halfway through, and cudaFree waits for the whole device,
// which stalls an assembly running on another stream.  bs2e_rk_get_batch_static
// does the same lookup through one file-scope device array instead:
//   - capacity kRkStaticMaxKeys keys per call (1.125 MiB per GPU that loads
//     the library, held until the process exits);
//   - bs2e_create resolves the array on the handle's device: it looks up the
//     array's device address with cudaGetSymbolAddress (that device current)
//     and loads the lookup kernel, so the module that holds the array is
//     resident before the caller fills HBM (under lazy module loading the
//     array would otherwise be reserved only at the first lookup).  The
//     lookup itself repeats that set-up when it finds none for its device;
//   - the address is valid for the device's current primary context: each
//     bs2e_create looks it up again, and a handle does not outlive a
//     cudaDeviceReset of its device;
//   - every call on a device uses the same array and leaves its contents
//     there: keys and values of the last call remain, nothing needs clearing
//     because each call overwrites exactly the part it reads;
//   - calls whose GPU work overlaps (several threads, several handles on one
//     device, or streams not ordered with each other) race on the array.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "bs2e_internal.h"

namespace bs2e {
namespace {

constexpr int64_t kRkStaticMaxKeys = 4096;
constexpr size_t kKeyBytes = (size_t)kRkStaticMaxKeys * 4 * sizeof(int64_t);      // 128 KiB
constexpr size_t kValBytes = (size_t)kRkStaticMaxKeys * kMaxK1 * sizeof(double);  // 1 MiB

// The scratch: keys (4 x int64 per key) followed by values (max_k+1 doubles per key).
static __device__ __align__(256) unsigned char g_rk_scratch[kKeyBytes + kValBytes];

// Device address of g_rk_scratch per device, looked up once per device.
std::mutex g_mu;
void *g_addr[64] = {nullptr};

// Same lookup as k_rk_gather, reading keys from and writing values to the scratch.
__global__ void k_rk_gather_static(const double *__restrict__ R, const float2 *__restrict__ Rf,
                                   const int *__restrict__ Rexp, int k, int K1, int N,
                                   int64_t tile, int64_t n, const int64_t *__restrict__ keys,
                                   double *__restrict__ vals) {
    const int W = 2 * k - 1;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * K1;
         e += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = e / K1;
        int kk = (int)(e - i * K1);
        int64_t a = keys[4 * i] - 1, b = keys[4 * i + 1] - 1, c = keys[4 * i + 2] - 1,
                d = keys[4 * i + 3] - 1;
        double v = 0.0;
        if (a >= 0 && a < N && b >= 0 && b < N && c >= 0 && c < N && d >= 0 && d < N &&
            c - a < k && a - c < k && d - b < k && b - d < k) {
            int dc = (int)(c - a) + k - 1, dd = (int)(d - b) + k - 1;
            size_t t = (size_t)(a * N + b);
            size_t o = t * tile + ((size_t)kk * W + dc) * W + dd;
            if (R) {
                v = R[o];
            } else {
                float2 x = Rf[o];
                int ex = Rexp[t * K1 + kk];
                double scale = __longlong_as_double((long long)(1023 - kRkBias + ex) << 52);
                v = ((double)x.x + (double)x.y) * scale;
            }
        }
        vals[e] = v;
    }
}

}  // namespace

// Looks up the scratch's device address on `device` (made current here) and
// loads the lookup kernel; refresh = true repeats the lookup when an address
// is cached already (a new handle may live in a new primary context).
cudaError_t noalloc_prepare(int device, bool refresh) {
    if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> g(g_mu);
    if (g_addr[device] && !refresh) return cudaSuccess;
    cudaError_t e = cudaSetDevice(device);
    void *p = nullptr;
    if (e == cudaSuccess) e = cudaGetSymbolAddress(&p, g_rk_scratch);
    cudaFuncAttributes fa;
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_rk_gather_static);
    if (e == cudaSuccess && !p) e = cudaErrorInvalidSymbol;
    g_addr[device] = (e == cudaSuccess) ? p : nullptr;
    return e;
}

}  // namespace bs2e

using namespace bs2e;

extern "C" BS2E_API bs2e_status bs2e_rk_get_batch_static(bs2e_handle *h, int64_t n,
                                                         const int64_t *keys, double *vals) {
    if (!h || n < 0 || (n > 0 && (!keys || !vals))) return BS2E_ERR_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    if (n > kRkStaticMaxKeys) {
        h->err = "bs2e_rk_get_batch_static: " + std::to_string(n) +
                 " keys requested, the static scratch holds at most " +
                 std::to_string(kRkStaticMaxKeys);
        return BS2E_ERR_ARG;
    }
    if (!h->d_R && !h->d_Rf) {
        h->err = "bs2e_rk has not run";
        return BS2E_ERR_STATE;
    }
    if (h->device < 0 || h->device >= 64) {
        h->err = "device ordinal out of range for the static scratch";
        return BS2E_ERR_ARG;
    }
    // set up (normally done by bs2e_create) before the n == 0 return, so an
    // empty call also leaves the array resolved
    cudaError_t e = cudaSetDevice(h->device);
    if (e == cudaSuccess) e = noalloc_prepare(h->device, false);
    void *base = nullptr;
    if (e == cudaSuccess) {
        std::lock_guard<std::mutex> g(g_mu);
        base = g_addr[h->device];
        if (!base) e = cudaErrorInvalidSymbol;
    }
    if (e == cudaSuccess && n == 0) return BS2E_OK;
    int64_t *d_keys = (int64_t *)base;
    double *d_vals = (double *)((unsigned char *)base + kKeyBytes);
    const Radial &g = h->g;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_keys, keys, sizeof(int64_t) * 4 * n, cudaMemcpyHostToDevice,
                            h->stream);
    if (e == cudaSuccess) {
        int64_t work = n * g.K1;
        unsigned grid = (unsigned)std::min<int64_t>((work + 255) / 256, 152 * 8);
        k_rk_gather_static<<<grid, 256, 0, h->stream>>>(h->d_R, h->d_Rf, h->d_Rexp, g.k, g.K1,
                                                         g.N, g.tile, n, d_keys, d_vals);
        h->launches++;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(vals, d_vals, sizeof(double) * n * g.K1, cudaMemcpyDeviceToHost,
                            h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
        h->err = std::string("bs2e_rk_get_batch_static: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? BS2E_ERR_NOMEM : BS2E_ERR_CUDA;
    }
    return BS2E_OK;
}
