// FP64 reprojection cost of a BAL problem without any device allocation.
//
// Some callers cannot let this library allocate device memory: a host
// framework that owns the whole device-memory budget through its own pool and
// hands libraries only the buffers it allocated, or a per-frame tracking loop
// that must not call cudaMalloc / cudaFree because those calls synchronise the
// device and stall the loop. For them, gba_cost_noalloc evaluates the same
// FP64 sum of squared Snavely residuals as the cost kernel of the solver
// (edge.cu, cost_f64), with its per-block partial sums kept in a fixed
// file-scope device array instead of caller- or solver-allocated scratch.
//
// The array (kCostScratchChunks partial sums and as many partial counts,
// 512 KiB) lives in every device that loads the library until the process
// exits. It is shared by every call: a call writes every slot it later reads,
// so nothing needs clearing between calls, but calls that overlap on the GPU
// (concurrent streams, or several host threads) race on it and must be
// serialised by the caller. Host code reaches the array only through the
// address cudaGetSymbolAddress returns for the current device (the symbol
// itself is a host-side stand-in); the first call on each device looks that
// address up, so that first call should come before any stream capture. The
// address is cached per device ordinal for the life of the process: it is
// stale after cudaDeviceReset destroys the device's primary context, and the
// entry point must not be called on that device after such a reset. The
// observation indices are not range-checked (the call receives no camera or
// point counts): they must lie inside the caller's arrays.

#include <mutex>

#include "camera_model.cuh"
#include "common.cuh"
#include "noalloc.hpp"

namespace gba {
namespace {

constexpr int kCostThreads = 256;
constexpr int kCostPerThread = 8;
constexpr int kCostChunk = kCostThreads * kCostPerThread;  // observations per CTA
constexpr int kCostScratchChunks = 32768;                  // -> at most 67,108,864 observations

// [0, kCostScratchChunks): per-chunk SSE; [kCostScratchChunks, 2 kCostScratchChunks):
// per-chunk count of non-finite residuals (exact in FP64 below 2^53).
static __device__ __align__(256) double g_cost_scratch[2 * kCostScratchChunks];

__global__ void __launch_bounds__(kCostThreads) cost_chunk_kernel(const double* __restrict__ cams,
                                                                 const double* __restrict__ pts,
                                                                 const int* __restrict__ oc, const int* __restrict__ op,
                                                                 const double* __restrict__ px, int E,
                                                                 double* __restrict__ scratch) {
    __shared__ double red[kCostThreads / 32];
    const long long base = static_cast<long long>(blockIdx.x) * kCostChunk;
    double sse = 0.0, bad = 0.0;
#pragma unroll 1
    for (int k = 0; k < kCostPerThread; ++k) {
        const long long e = base + k * kCostThreads + threadIdx.x;
        if (e >= E) break;
        double cam[9], X[3], obs[2], r[2];
        const double* c = cams + 9ll * oc[e];
        const double* x = pts + 3ll * op[e];
#pragma unroll
        for (int i = 0; i < 9; ++i) cam[i] = c[i];
#pragma unroll
        for (int i = 0; i < 3; ++i) X[i] = x[i];
        obs[0] = px[2 * e];
        obs[1] = px[2 * e + 1];
        model::residual(cam, X, obs, r);
        if (isfinite(r[0]) && isfinite(r[1]))
            sse += r[0] * r[0] + r[1] * r[1];
        else
            bad += 1.0;
    }
    const double s = block_sum<kCostThreads>(sse, red);
    const double b = block_sum<kCostThreads>(bad, red);
    if (threadIdx.x == 0) {
        scratch[blockIdx.x] = s;
        scratch[kCostScratchChunks + blockIdx.x] = b;
    }
}

__global__ void __launch_bounds__(256) cost_chunk_finalize(const double* __restrict__ scratch, int nchunks,
                                                          double* __restrict__ out_sse,
                                                          unsigned long long* __restrict__ out_bad) {
    __shared__ double red[8];
    double s = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < nchunks; i += 256) {
        s += scratch[i];
        b += scratch[kCostScratchChunks + i];
    }
    const double ts = block_sum<256>(s, red);
    const double tb = block_sum<256>(b, red);
    if (threadIdx.x == 0) {
        *out_sse = ts;
        if (out_bad) *out_bad = static_cast<unsigned long long>(tb);
    }
}

constexpr int kMaxDevices = 64;
std::mutex g_addr_mutex;
double* g_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once
// per device, with that device current; valid until the device's primary
// context is destroyed, e.g. by cudaDeviceReset).
double* scratch_address() {
    int dev = 0;
    GBA_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) throw std::invalid_argument("device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    if (!g_addr[dev]) {
        void* p = nullptr;
        GBA_CUDA_CHECK(cudaGetSymbolAddress(&p, g_cost_scratch));
        g_addr[dev] = static_cast<double*>(p);
    }
    return g_addr[dev];
}

}  // namespace

long long cost_noalloc_max_observations() { return static_cast<long long>(kCostScratchChunks) * kCostChunk; }

void cost_noalloc(const double* cams, const double* pts, const int* oc, const int* op, const double* px, int E,
                  double* out_sse, unsigned long long* out_bad, cudaStream_t s) {
    if (E < 0) throw std::invalid_argument("negative observation count");
    if (E > cost_noalloc_max_observations())
        throw std::invalid_argument("gba_cost_noalloc: num_observations " + std::to_string(E) +
                                    " exceeds the fixed scratch limit of " +
                                    std::to_string(cost_noalloc_max_observations()) + " observations");
    double* scratch = scratch_address();
    const int nchunks = ceil_div(E, kCostChunk);
    if (nchunks > 0) {
        cost_chunk_kernel<<<nchunks, kCostThreads, 0, s>>>(cams, pts, oc, op, px, E, scratch);
        GBA_LAUNCH_CHECK();
    }
    cost_chunk_finalize<<<1, 256, 0, s>>>(scratch, nchunks, out_sse, out_bad);
    GBA_LAUNCH_CHECK();
}

}  // namespace gba
